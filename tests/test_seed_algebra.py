"""The block algebra and the scratch bound of the seed inverse (spd_inverse_seed in
csrc/spd_inverse.cu), restated in NumPy with exact FP64 products:

    G = [A B; B^T C]:  W = A^-1 B,  S = C - B^T W,  V = W S^-1,
    G^-1 = [A^-1 + V W^T, -V; -V^T, S^-1],

split at m1 = m/2 rounded up to a multiple of 128, recursing on A and S down to blocks
of at most 1,024 rows.  The kernel keeps W and V of every level in one scratch block of
m^2 doubles (W, V at its start, the inner levels after them); the bound below is what
makes that block large enough for every size."""
from functools import lru_cache

import numpy as np

MT = 128
BASE = 1024


def split(m):
    m1 = (m // 2 + MT - 1) // MT * MT
    return m1, m - m1


@lru_cache(None)
def scratch_doubles(m):
    """Doubles of scratch the recursion touches (W and V of this level, then the larger of
    the two inner recursions, which run one after the other on the same region)."""
    if m <= BASE:
        return 0
    m1, m2 = split(m)
    return 2 * m1 * m2 + max(scratch_doubles(m1), scratch_doubles(m2))


def seed_inverse(G, base=BASE):
    m = G.shape[0]
    if m <= base:
        return np.linalg.inv(G)
    m1, _ = split(m)
    A, B, C = G[:m1, :m1], G[:m1, m1:], G[m1:, m1:]
    XA = seed_inverse(A, base)
    W = XA @ B
    S = C - B.T @ W
    XS = seed_inverse(0.5 * (S + S.T), base)
    V = W @ XS
    X = np.empty_like(G)
    X[:m1, :m1] = XA + V @ W.T
    X[:m1, m1:] = -V
    X[m1:, :m1] = -V.T
    X[m1:, m1:] = XS
    return X


def test_block_recursion_inverts_an_nnls_like_matrix():
    rng = np.random.default_rng(3)
    for m, base in ((700, 200), (1500, 300)):
        U = rng.random((m, 2 * m)) ** 4          # non-negative rows, like a library
        G = U @ U.T + np.eye(m) * np.mean(np.sum(U * U, 1)) / U.shape[1]
        X = seed_inverse(G, base)
        assert np.linalg.norm(np.eye(m) - G @ X) < 1e-9


def test_scratch_fits_in_m_squared_and_blocks_fit_the_base():
    worst = 0.0
    for m in range(1, 60001, 7):
        worst = max(worst, scratch_doubles(m) / (m * m))
        if m > BASE:
            m1, m2 = split(m)
            assert 0 < m1 < m and 0 < m2 < m
    assert worst < 0.7


def test_config_sizes_split_into_blocks_below_the_base():
    def blocks(m, out):
        if m <= BASE:
            out.append(m)
            return
        m1, m2 = split(m)
        blocks(m1, out)
        blocks(m2, out)

    for m, n_blocks in ((6608, 8), (23884, 32)):
        b = []
        blocks(m, b)
        assert len(b) == n_blocks and sum(b) == m and max(b) <= BASE
