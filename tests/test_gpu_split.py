"""Split (Ozaki) tensor-core products through the C ABI, against FP64 products.

Each row of A and column of B keeps 31 (4 slices) or 39 (5 slices) bits below
its largest magnitude, and slice pairs up to s + t = 6 are formed, so

  |C - AB|_ij <= 2^-bits (max_k |A_ik| sum_k |B_kj| + max_k |B_kj| sum_k |A_ik|)
                 + 2^-34 K max_k |A_ik| max_k |B_kj|

up to a small factor (the second term: the dropped pairs s + t = 7, and the FP32
rounding of the levels >= 4, each a few 2^-40 of K max|A| max|B| once the
scales 2^e <= 2 max are counted); the tests allow a factor 8 on the first term."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def K():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from schwarmax_gb300 import kernels
    return kernels


def _bound(A, B, bits, second=2.0 ** -34):
    """Right-hand side of the error bound above (factor 8 on the slicing term)."""
    ra = A.abs().amax(1, keepdim=True)            # (M, 1)
    cb = B.abs().amax(0, keepdim=True)            # (1, N)
    t1 = ra * B.abs().sum(0, keepdim=True) + A.abs().sum(1, keepdim=True) * cb
    return 8 * 2.0 ** -bits * t1 + second * A.shape[1] * ra * cb


def _check(C, A, B, bits, second=2.0 ** -34):
    ref = A @ B
    bound = _bound(A, B, bits, second)
    ratio = ((C - ref).abs() / bound.clamp_min(1e-300)).max().item()
    assert ratio <= 1.0, ratio


@pytest.mark.parametrize("M,N,Kd,sa,sb", [
    (300, 100, 1000, 4, 4),        # one vector tile, k inside one exact chunk pair
    (1000, 112, 20000, 4, 4),      # k across chunks and across the int32 output flush
    (700, 100, 3000, 5, 4),        # G^-1 style operand with 5 slices
    (500, 300, 2500, 4, 4),        # several 128-wide column tiles
    (260, 260, 9000, 5, 5),
    (600, 100, 5000, 5, 5),        # 64-wide column tiles with five exact levels (G^-1 E)
])
def test_split_gemm_error_bound(K, M, N, Kd, sa, sb):
    g = torch.Generator(device="cuda").manual_seed(M + N + Kd)
    A = torch.randn(M, Kd, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(Kd, N, dtype=torch.float64, device="cuda", generator=g)
    # wide dynamic range inside rows and columns
    A = A * torch.exp(3 * torch.randn(M, Kd, dtype=torch.float64, device="cuda", generator=g))
    B[:, 0] = 0.0                  # an all-zero column
    C = K.split_gemm(A, B, sa, sb)
    # 5 x 5 slices with N <= 128 run on 64-wide tiles with five exact levels:
    # only the slicing of the inputs remains
    exact5 = sa == 5 and sb == 5 and N <= 128
    _check(C, A, B, 31 if min(sa, sb) == 4 else 39, 2.0 ** -60 if exact5 else 2.0 ** -34)
    assert torch.all(C[:, 0] == 0)


def test_split_gemm_seven_slices(K):
    """7 x 7 slices, levels up to 8 and four exact levels (the products of the
    Newton-Schulz inverse): checked against a long-double reference, since an
    FP64 product is less accurate than the split one."""
    rng = np.random.default_rng(7)
    M, N, Kd = 256, 192, 3000
    A = rng.standard_normal((M, Kd)) * np.exp(2 * rng.standard_normal((M, Kd)))
    B = rng.standard_normal((Kd, N))
    ref = (A.astype(np.longdouble) @ B.astype(np.longdouble))
    C = K.split_gemm(torch.tensor(A, device="cuda"), torch.tensor(B, device="cuda"), 7, 7).cpu().numpy()
    ra = np.abs(A).max(1, keepdims=True)
    cb = np.abs(B).max(0, keepdims=True)
    bound = 8 * 2.0 ** -55 * (ra * np.abs(B).sum(0, keepdims=True) + np.abs(A).sum(1, keepdims=True) * cb) \
        + 2.0 ** -52 * Kd * ra * cb
    err = np.abs((C.astype(np.longdouble) - ref).astype(np.float64))
    assert (err / bound).max() <= 1.0, (err / bound).max()
    # and it is far below the error of the 5 x 5 product
    C5 = K.split_gemm(torch.tensor(A, device="cuda"), torch.tensor(B, device="cuda"), 5, 5).cpu().numpy()
    err5 = np.abs((C5.astype(np.longdouble) - ref).astype(np.float64))
    assert err.max() < err5.max() / 100


@pytest.mark.parametrize("m,sl", [(700, 4), (1000, 5)])
def test_split_gemm_lower_tiles(K, m, sl):
    """Symmetric products over the lower-triangle tiles only (the Gram matrix)."""
    g = torch.Generator(device="cuda").manual_seed(m)
    U = torch.rand(m, 3000, dtype=torch.float64, device="cuda", generator=g) ** 3
    Ut = U.t().contiguous()
    C = K.split_gemm(U, Ut, sl, sl, lower=True)
    ref = U @ Ut
    tiles = torch.arange(m, device="cuda") // 128
    low = tiles[:, None] >= tiles[None, :]
    assert torch.all(C[~low] == 0)
    bound = _bound(U, Ut, 31 if sl == 4 else 39)
    ratio = (((C - ref).abs() / bound)[low]).max().item()
    assert ratio <= 1.0, ratio


def test_split_gemm_integers_exact(K):
    """Integers in [-64, 64] are single slices (scaled by 2^(7-e) they stay
    integers of at most 128), so only level-2 sums occur and they are exact."""
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randint(-64, 65, (256, 4096), device="cuda", generator=g).double()
    B = torch.randint(-64, 65, (4096, 96), device="cuda", generator=g).double()
    A[0, :] = 64.0                 # the largest slice values in every product of row 0
    B[:, 1] = -64.0
    C = K.split_gemm(A, B)
    assert torch.equal(C, A @ B)


def test_split_gemm_nonnegative_library_shape(K):
    """Shapes and value ranges of the NNLS products: U (m x n, non-negative,
    sparse) times a vector block, and the Gram-like U U^T."""
    g = torch.Generator(device="cuda").manual_seed(5)
    m, n, B = 900, 2048, 100
    U = torch.rand(m, n, dtype=torch.float64, device="cuda", generator=g) ** 4
    U[torch.rand(m, n, device="cuda", generator=g) < 0.7] = 0.0
    U = U.float().double()         # float library values
    D = torch.rand(n, B, dtype=torch.float64, device="cuda", generator=g) - 0.2
    _check(K.split_gemm(U, D), U, D, 31)
    Ut = U.t().contiguous()
    _check(K.split_gemm(U, Ut), U, Ut, 31)


@pytest.mark.parametrize("m", [5, 200, 777])
def test_spd_inverse_seed(m):
    """The FP32 blocked Gauss-Jordan inverse that seeds Newton-Schulz: residual
    ||I - G X||_F far below 1 for a matrix with the NNLS's structure (c I + U U^T)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import kernels
    g = torch.Generator(device="cuda").manual_seed(m)
    U = torch.randn(m, 2 * m + 3, generator=g, device="cuda", dtype=torch.float64)
    U = U * torch.logspace(0, 2, m, device="cuda", dtype=torch.float64)[:, None]    # uneven row scales
    G = (U @ U.t() + (U * U).sum() / U.shape[1] * torch.eye(m, device="cuda", dtype=torch.float64)).contiguous()
    X = kernels.spd_inverse_f32(G).double()
    R = torch.eye(m, device="cuda", dtype=torch.float64) - G @ X
    assert float(torch.linalg.norm(R)) < 1e-2


@pytest.mark.parametrize("m", [300, 1500, 2900])
def test_spd_inverse_schur_seed(m):
    """The seed the mixed NNLS refines: Schur-complement recursion on split products with
    Gauss-Jordan blocks of up to 1,024 rows (one level at 1,500, two at 2,900).  It is
    exactly symmetric and as good as the FP32 Gauss-Jordan inverse of the whole matrix."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from schwarmax_gb300 import kernels
    g = torch.Generator(device="cuda").manual_seed(m)
    U = torch.rand(m, 2 * m + 3, generator=g, device="cuda", dtype=torch.float64) ** 4    # non-negative, like a library
    U = U * torch.logspace(0, 1, m, device="cuda", dtype=torch.float64)[:, None]
    G = (U @ U.t() + (U * U).sum() / U.shape[1] * torch.eye(m, device="cuda", dtype=torch.float64)).contiguous()
    eye = torch.eye(m, device="cuda", dtype=torch.float64)
    X = kernels.spd_inverse_seed(G)
    assert torch.equal(X, X.t())
    r_seed = float(torch.linalg.norm(eye - G @ X))
    r_gj = float(torch.linalg.norm(eye - G @ kernels.spd_inverse_f32(G).double()))
    assert r_seed < 1e-2 and r_seed < 4 * r_gj, (r_seed, r_gj)
