// Inverse of a symmetric positive definite matrix in FP32 by blocked Gauss-Jordan
// elimination without pivoting: the seed of the Newton-Schulz refinement of G^-1 in
// the mixed NNLS (it replaces the float Cholesky inverse the reference's
// jnp.linalg.cholesky step would suggest, nnls.py:121; only a residual well below 1
// is needed, Newton-Schulz supplies the accuracy).
//
// For every 64-wide block k of the (padded) matrix, in place:
//   P = A_kk^-1                       (one CTA, unblocked Gauss-Jordan in shared memory)
//   R_k: = P A_k:                     (row panel, into a buffer)
//   A_ij -= A_ik R_kj                 (i, j outside block k: 128 x 128 tiles, 8 x 8 per thread)
//   A_ik = -A_ik P,  A_kj = R_kj,  A_kk = P
// which leaves A^-1 after the last block.  2 m^3 flops on the FP32 pipe; the matrix
// is padded to a multiple of 64 with an identity block.
#include "smx_internal.cuh"
#include "split_gemm.cuh"

namespace smx {

constexpr int GJ_B = 64;      // elimination block
constexpr int GJ_T = 128;     // update tile

// unblocked Gauss-Jordan of the 64 x 64 diagonal block k (column-major, leading
// dimension ld), P written column-major 64 x 64.  256 threads on a 16 x 16 grid, each
// holding a 4 x 4 tile in registers (the pivot loop is unrolled, so every register
// index is static); per pivot the 16 threads on the pivot row and the 16 on the pivot
// column publish their parts through shared memory (double-buffered, one barrier per
// pivot).  Every update is s_rc - s_rk (s_kc / s_kk), in the order of the textbook form.
__global__ void __launch_bounds__(256) gj_diag_kernel(const float *__restrict__ A, int64_t ld, int64_t k0, float *P,
                                                      int *flag) {
    __shared__ float rowb[2][GJ_B], colb[2][GJ_B];
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    float a[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) a[i][j] = A[(k0 + 4 * tr + i) + ld * (k0 + 4 * tc + j)];
#pragma unroll
    for (int k = 0; k < GJ_B; ++k) {
        const int b = k & 1, kb = k >> 2, kr = k & 3;
        if (tr == kb) {
#pragma unroll
            for (int j = 0; j < 4; ++j) rowb[b][4 * tc + j] = a[kr][j];
        }
        if (tc == kb) {
#pragma unroll
            for (int i = 0; i < 4; ++i) colb[b][4 * tr + i] = a[i][kr];
        }
        __syncthreads();
        const float piv = rowb[b][k];
        if (!(piv > 0.0f)) {   // uniform: every thread read the same pivot
            if (threadIdx.x == 0) atomicExch(flag, 1);
            return;
        }
        const float ip = 1.0f / piv;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = 4 * tr + i;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * tc + j;
                float v;
                if (r == k) v = (c == k) ? ip : rowb[b][c] * ip;
                else if (c == k) v = -colb[b][r] * ip;
                else v = a[i][j] - colb[b][r] * (rowb[b][c] * ip);
                a[i][j] = v;
            }
        }
        // the next pivot writes the other buffers, so one barrier per pivot suffices
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) P[(4 * tr + i) + GJ_B * (4 * tc + j)] = a[i][j];
}

// R (64 x mp, row r at R + mp r) = P A[k block rows, :]; grid over 128-column tiles
__global__ void __launch_bounds__(256) gj_row_kernel(const float *__restrict__ A, int64_t ld, int64_t k0,
                                                     const float *__restrict__ P, float *R) {
    __shared__ float sp[GJ_B][GJ_B + 1];
    __shared__ float sa[GJ_B][GJ_T + 1];
    const int64_t j0 = (int64_t)blockIdx.x * GJ_T;
    for (int e = threadIdx.x; e < GJ_B * GJ_B; e += blockDim.x) sp[e % GJ_B][e / GJ_B] = P[e];
    for (int e = threadIdx.x; e < GJ_B * GJ_T; e += blockDim.x) {
        const int r = e % GJ_B, c = e / GJ_B;
        sa[r][c] = A[(k0 + r) + ld * (j0 + c)];
    }
    __syncthreads();
    // each thread: column c = tid % 128, rows r = tid / 128 + 2 q (consecutive threads
    // write consecutive columns of a row)
    const int c = threadIdx.x % GJ_T;
    for (int r = threadIdx.x / GJ_T; r < GJ_B; r += 2) {
        float acc = 0.f;
#pragma unroll 16
        for (int l = 0; l < GJ_B; ++l) acc += sp[r][l] * sa[l][c];
        R[(j0 + c) + ld * r] = acc;
    }
}

// A_ij -= A_ik R_kj for the 128 x 128 tile (blockIdx.x, blockIdx.y), skipping the
// rows and columns of block k.  Thread (tx, ty) of 16 x 16 owns rows 8 tx .. 8 tx + 7
// (contiguous, read and written as float4) of columns ty + 16 b, b < 8; both panels are
// staged in shared memory with coalesced loads (R row-major: R[j + ld l]).
__global__ void __launch_bounds__(256) gj_update_kernel(float *A, int64_t ld, int64_t k0, const float *__restrict__ R) {
    __shared__ __align__(16) float sc[GJ_B][GJ_T];   // sc[l][i]: A[i0 + i, k0 + l]
    __shared__ __align__(16) float sr[GJ_B][GJ_T];   // sr[l][j]: R[l, j0 + j]
    const int64_t i0 = (int64_t)blockIdx.x * GJ_T, j0 = (int64_t)blockIdx.y * GJ_T;
    for (int e = threadIdx.x; e < GJ_B * GJ_T / 4; e += blockDim.x) {
        const int i4 = e % (GJ_T / 4), l = e / (GJ_T / 4);
        *(float4 *)&sc[l][4 * i4] = *(const float4 *)&A[(i0 + 4 * i4) + ld * (k0 + l)];
        *(float4 *)&sr[l][4 * i4] = *(const float4 *)&R[(j0 + 4 * i4) + ld * l];
    }
    __syncthreads();
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
#pragma unroll 4
    for (int l = 0; l < GJ_B; ++l) {
        float ci[8], rj[8];
        const float4 c0 = *(const float4 *)&sc[l][8 * tx], c1 = *(const float4 *)&sc[l][8 * tx + 4];
        ci[0] = c0.x; ci[1] = c0.y; ci[2] = c0.z; ci[3] = c0.w;
        ci[4] = c1.x; ci[5] = c1.y; ci[6] = c1.z; ci[7] = c1.w;
#pragma unroll
        for (int b = 0; b < 8; ++b) rj[b] = sr[l][ty + 16 * b];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 8; ++b) acc[a][b] += ci[a] * rj[b];
    }
    const int64_t ib = i0 + 8 * tx;
    const bool rows_in_k = ib >= k0 && ib < k0 + GJ_B;   // 8-row groups lie inside or outside block k
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int64_t j = j0 + ty + 16 * b;
        if (rows_in_k || (j >= k0 && j < k0 + GJ_B)) continue;
        float4 *p = (float4 *)&A[ib + ld * j];
        float4 v0 = p[0], v1 = p[1];
        v0.x -= acc[0][b]; v0.y -= acc[1][b]; v0.z -= acc[2][b]; v0.w -= acc[3][b];
        v1.x -= acc[4][b]; v1.y -= acc[5][b]; v1.z -= acc[6][b]; v1.w -= acc[7][b];
        p[0] = v0;
        p[1] = v1;
    }
}

// A_ik = -A_ik P for the rows of a 128-row tile outside block k; the tile that holds
// block k also writes A_kk = P.  The row panel A_kj = R_kj is copied by gj_copy_kernel.
__global__ void __launch_bounds__(256) gj_col_kernel(float *A, int64_t ld, int64_t k0, const float *__restrict__ P) {
    __shared__ float sp[GJ_B][GJ_B + 1];
    __shared__ float sa[GJ_T][GJ_B + 1];
    const int64_t i0 = (int64_t)blockIdx.x * GJ_T;
    for (int e = threadIdx.x; e < GJ_B * GJ_B; e += blockDim.x) sp[e % GJ_B][e / GJ_B] = P[e];
    for (int e = threadIdx.x; e < GJ_T * GJ_B; e += blockDim.x) {
        const int i = e % GJ_T, l = e / GJ_T;
        sa[i][l] = A[(i0 + i) + ld * (k0 + l)];
    }
    __syncthreads();
    const int i = threadIdx.x % GJ_T;
    const int64_t gi = i0 + i;
    const bool inblk = gi >= k0 && gi < k0 + GJ_B;
    for (int c = threadIdx.x / GJ_T; c < GJ_B; c += 2) {
        float v;
        if (inblk) {
            v = sp[gi - k0][c];
        } else {
            float acc = 0.f;
#pragma unroll 16
            for (int l = 0; l < GJ_B; ++l) acc += sa[i][l] * sp[l][c];
            v = -acc;
        }
        A[gi + ld * (k0 + c)] = v;
    }
}

__global__ void gj_copy_kernel(float *A, int64_t ld, int64_t k0, const float *__restrict__ R, int64_t mp) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < GJ_B * mp; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e % GJ_B, j = e / GJ_B;
        if (j >= k0 && j < k0 + GJ_B) continue;
        A[(k0 + r) + ld * j] = R[j + ld * r];
    }
}

// padded copy: Ap (mp x mp) = G (m x m, double) in float, identity on the padding
__global__ void gj_pad_kernel(const double *__restrict__ G, int64_t m, float *Ap, int64_t mp) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mp * mp; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e % mp, c = e / mp;
        Ap[e] = (r < m && c < m) ? (float)G[r + m * c] : (r == c ? 1.0f : 0.0f);
    }
}

int64_t spd_inverse_padded(int64_t m) { return (m + GJ_T - 1) / GJ_T * GJ_T; }

size_t spd_inverse_workspace(int64_t m) {
    const int64_t mp = spd_inverse_padded(m);
    return (size_t)(mp * mp + GJ_B * GJ_B + GJ_B * mp) * sizeof(float) + 256;
}

// Ap (mp x mp float, padded by gj_pad_kernel) is overwritten by its inverse.
// ws: GJ_B^2 + GJ_B mp floats of scratch plus an int flag (set when a pivot is not positive).
int spd_inverse_inplace(float *Ap, int64_t mp, float *ws, int *flag, cudaStream_t s) {
    float *P = ws, *R = ws + GJ_B * GJ_B;
    const unsigned tiles = (unsigned)(mp / GJ_T);
    for (int64_t k0 = 0; k0 < mp; k0 += GJ_B) {
        gj_diag_kernel<<<1, 256, 0, s>>>(Ap, mp, k0, P, flag);
        gj_row_kernel<<<tiles, 256, 0, s>>>(Ap, mp, k0, P, R);
        gj_update_kernel<<<dim3(tiles, tiles), 256, 0, s>>>(Ap, mp, k0, R);
        gj_col_kernel<<<tiles, 256, 0, s>>>(Ap, mp, k0, P);
        gj_copy_kernel<<<(unsigned)((GJ_B * mp + 255) / 256), 256, 0, s>>>(Ap, mp, k0, R, mp);
        count_launch(5);
    }
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

// ------------------------------------------------------------ recursive seed
// G^-1 of a symmetric positive definite G by block elimination on Schur complements,
//   G = [A B; B^T C]:  X_A = A^-1,  W = X_A B,  S = C - B^T W,  X_S = S^-1,
//   V = W X_S,  G^-1 = [X_A + V W^T, -V; -V^T, X_S],
// with A^-1 and S^-1 by the same rule down to blocks of at most kSeedBaseRows rows, which
// the FP32 Gauss-Jordan above inverts and one Newton-Schulz step (R = I - A X,
// X += X R) refines.  Every product runs on the split tensor-core kernel with 5 slices
// and pairs s + t <= 6 (39 bits of every row's and column's largest magnitude); the
// products are about m^3 flops per slice pair in all.  The Schur complements of an SPD
// matrix are SPD, so no pivoting is needed.  The result is exactly symmetric (the
// symmetric products are formed on their lower tiles and mirrored).

namespace {

constexpr int kSeedSlices = 5;
constexpr int kSeedLevels = 6;        // slice pairs s + t <= 6

__device__ __forceinline__ double exp2i(int p) { return __longlong_as_double((long long)(1023 + p) << 52); }

// out = beta out + alpha C for the product C (M x N) in T, R (leading dimension M, row
// exponents eA, column exponents eB, T in units of 2^-t_shift).  lower: C symmetric,
// formed on the lower tiles only; every element above the diagonal takes its mirror's
// value, so the result is exactly symmetric.
__global__ void seed_combine_kernel(const unsigned long long *__restrict__ T, const float *__restrict__ R,
                                    const int32_t *__restrict__ eA, const int32_t *__restrict__ eB, int t_shift,
                                    int64_t M, int64_t N, double alpha, double beta, double *out, int64_t ldo,
                                    int lower) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < M * N; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k % M, j = k / M;
        int64_t ti = i, tj = j;
        if (lower && j > i) {   // (j, i) lies in a lower tile
            ti = j;
            tj = i;
        }
        const int64_t idx = ti + M * tj;
        const double c = ((double)(long long)T[idx] * exp2i(-t_shift) + (double)R[idx]) * exp2i(eA[ti] + eB[tj] - 14);
        double *o = out + i + ldo * j;
        *o = (beta != 0.0 ? beta * *o : 0.0) + alpha * c;
    }
}

__global__ void seed_clear_kernel(unsigned long long *T, float *R, int64_t count) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        T[k] = 0ull;
        R[k] = 0.0f;
    }
}

// X_12 = -V, X_21 = -V^T (V is m1 x m2 with leading dimension m1)
__global__ void seed_offdiag_kernel(const double *__restrict__ V, int64_t m1, int64_t m2, double *X, int64_t ld) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m1 * m2; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k % m1, j = k / m1;
        const double v = -V[k];
        X[i + ld * (m1 + j)] = v;
        X[(m1 + j) + ld * i] = v;
    }
}

// the m x m block at X (leading dimension ld) as a padded float matrix, identity on the padding
__global__ void seed_pad_kernel(const double *__restrict__ X, int64_t ld, int64_t m, float *Ap, int64_t mp) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mp * mp; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e % mp, c = e / mp;
        Ap[e] = (r < m && c < m) ? (float)X[r + ld * c] : (r == c ? 1.0f : 0.0f);
    }
}

// B (m x m, leading dimension m) = the block at X (leading dimension ld); I = identity in R
__global__ void seed_copy_kernel(const double *__restrict__ X, int64_t ld, int64_t m, double *B, double *R) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * m; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e % m, c = e / m;
        B[e] = X[r + ld * c];
        R[e] = r == c ? 1.0 : 0.0;
    }
}

// the block back in double, symmetrised
__global__ void seed_unpad_kernel(const float *__restrict__ Ap, int64_t mp, double *X, int64_t ld, int64_t m) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * m; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e % m, c = e / m;
        X[r + ld * c] = 0.5 * ((double)Ap[r + mp * c] + (double)Ap[c + mp * r]);
    }
}

inline unsigned seed_grid(int64_t count) {
    int64_t g = (count + 255) / 256;
    if (g > 152 * 32) g = 152 * 32;
    return (unsigned)(g < 1 ? 1 : g);
}

// out = beta out + alpha A_op B_op^T with A_op(i, k) = a[i asr + k asc] (M x K) and
// B_op(j, k) = b[j bsr + k bsc] (N x K)
int seed_product(const SeedWorkspace &w, const double *a, int64_t asr, int64_t asc, const double *b, int64_t bsr,
                 int64_t bsc, int64_t M, int64_t N, int64_t K, bool lower, double alpha, double beta, double *out,
                 int64_t ldo, cudaStream_t s) {
    split::Operand A = split::make_operand(M, K, split::MT, kSeedSlices);
    split::Operand B = split::make_operand(N, K, split::MT, kSeedSlices);
    A.slices = w.a_slices;
    A.expo = w.a_expo;
    B.slices = w.b_slices;
    B.expo = w.b_expo;
    int st;
    if ((st = split::slice_rows<double>(a, asr, asc, A, w.rowmax, s))) return st;
    if ((st = split::slice_rows<double>(b, bsr, bsc, B, w.rowmax, s))) return st;
    split::Acc acc{w.T, w.R, M};
    if ((st = split::gemm(A, B, acc, lower, w.err, s, kSeedLevels))) return st;
    seed_combine_kernel<<<seed_grid(M * N), 256, 0, s>>>(w.T, w.R, A.expo, B.expo, 8 * (split::exact_levels(A, B) - 1),
                                                         M, N, alpha, beta, out, ldo, lower ? 1 : 0);
    seed_clear_kernel<<<seed_grid(M * N), 256, 0, s>>>(w.T, w.R, M * N);
    count_launch(2);
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

}  // namespace

// In place: the m x m block at X (leading dimension ld) holds G on entry and the seed
// of G^-1 on return.  scratch: the W and V blocks of every level (at most 0.7 m^2 doubles).
int spd_inverse_seed(double *X, int64_t ld, int64_t m, double *scratch, const SeedWorkspace &w, cudaStream_t s) {
    int st;
    if (m <= kSeedBaseRows) {
        const int64_t mp = spd_inverse_padded(m);
        double *A0 = w.base, *R = w.base + m * m;
        seed_copy_kernel<<<seed_grid(m * m), 256, 0, s>>>(X, ld, m, A0, R);
        seed_pad_kernel<<<seed_grid(mp * mp), 256, 0, s>>>(X, ld, m, w.gp, mp);
        count_launch(2);
        if ((st = spd_inverse_inplace(w.gp, mp, w.gjws, w.flag, s))) return st;
        seed_unpad_kernel<<<seed_grid(m * m), 256, 0, s>>>(w.gp, mp, X, ld, m);
        count_launch();
        if ((st = seed_product(w, A0, 1, m, X, ld, 1, m, m, m, false, -1.0, 1.0, R, m, s))) return st;   // R = I - A X
        if ((st = seed_product(w, X, 1, ld, R, m, 1, m, m, m, true, 1.0, 1.0, X, ld, s))) return st;     // X += X R
        SMX_TRY_CUDA(cudaGetLastError());
        return SMX_OK;
    }
    const int64_t m1 = (m / 2 + split::MT - 1) / split::MT * split::MT, m2 = m - m1;
    double *A = X, *B = X + ld * m1, *C = X + m1 + ld * m1;
    double *W = scratch, *V = scratch + m1 * m2, *inner = scratch + 2 * m1 * m2;
    if ((st = spd_inverse_seed(A, ld, m1, inner, w, s))) return st;                                    // X_A
    if ((st = seed_product(w, A, 1, ld, B, ld, 1, m1, m2, m1, false, 1.0, 0.0, W, m1, s))) return st;   // W = X_A B
    if ((st = seed_product(w, B, ld, 1, W, m1, 1, m2, m2, m1, true, -1.0, 1.0, C, ld, s))) return st;   // S = C - B^T W
    if ((st = spd_inverse_seed(C, ld, m2, inner, w, s))) return st;                                    // X_S
    if ((st = seed_product(w, W, 1, m1, C, ld, 1, m1, m2, m2, false, 1.0, 0.0, V, m1, s))) return st;   // V = W X_S
    if ((st = seed_product(w, V, 1, m1, W, 1, m1, m1, m1, m2, true, 1.0, 1.0, A, ld, s))) return st;    // X_A += V W^T
    seed_offdiag_kernel<<<seed_grid(m1 * m2), 256, 0, s>>>(V, m1, m2, X, ld);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

}  // namespace smx

using namespace smx;

extern "C" int smx_spd_inverse_f32_workspace_size(int64_t m, size_t *bytes) {
    if (m < 1 || !bytes) return set_error(SMX_ERR_ARGUMENT, "smx_spd_inverse_f32_workspace_size: bad argument");
    const int64_t mp = spd_inverse_padded(m);
    *bytes = (size_t)mp * mp * sizeof(float) + spd_inverse_workspace(m) + 256;
    return SMX_OK;
}

extern "C" int smx_spd_inverse_f32(const double *G, int64_t m, float *Xinv, void *workspace, size_t workspace_bytes,
                                   void *stream) {
    if (m < 1 || m > 46340 || !G || !Xinv || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_spd_inverse_f32: bad argument");
    size_t need = 0;
    int st = smx_spd_inverse_f32_workspace_size(m, &need);
    if (st) return st;
    if (workspace_bytes < need) return set_error(SMX_ERR_WORKSPACE, "smx_spd_inverse_f32: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t mp = spd_inverse_padded(m);
    float *Ap = (float *)workspace;
    float *ws = Ap + mp * mp;
    int *flag = (int *)(ws + GJ_B * GJ_B + GJ_B * mp);
    SMX_TRY_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    gj_pad_kernel<<<4864, 256, 0, s>>>(G, m, Ap, mp);
    count_launch();
    if ((st = spd_inverse_inplace(Ap, mp, ws, flag, s))) return st;
    SMX_TRY_CUDA(cudaMemcpy2DAsync(Xinv, m * sizeof(float), Ap, mp * sizeof(float), m * sizeof(float), m,
                                   cudaMemcpyDeviceToDevice, s));
    int hflag = 0;
    SMX_TRY_CUDA(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (hflag) return set_error(SMX_ERR_NUMERIC, "smx_spd_inverse_f32: a pivot was not positive");
    return SMX_OK;
}

namespace {
struct SeedLayout {
    split::Operand a, b;
    size_t a_sl, a_e, b_sl, b_e, T, R, rowmax, scratch, base, gp, gjws, err, total;
};
SeedLayout seed_layout(int64_t m) {
    SeedLayout L;
    L.a = split::make_operand(m, m, split::MT, kSeedSlices);
    L.b = split::make_operand(m, m, split::MT, kSeedSlices);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    const int64_t mb = m < kSeedBaseRows ? m : kSeedBaseRows, mp = spd_inverse_padded(mb);
    L.a_sl = take(L.a.slice_bytes());
    L.a_e = take(L.a.row_tiles * split::MT * sizeof(int32_t));
    L.b_sl = take(L.b.slice_bytes());
    L.b_e = take(L.b.row_tiles * split::MT * sizeof(int32_t));
    L.T = take((size_t)m * m * sizeof(unsigned long long));
    L.R = take((size_t)m * m * sizeof(float));
    L.rowmax = take((size_t)m * sizeof(unsigned long long));
    L.scratch = take((size_t)m * m * sizeof(double));
    L.base = take((size_t)2 * mb * mb * sizeof(double));
    L.gp = take((size_t)mp * mp * sizeof(float));
    L.gjws = take(spd_inverse_workspace(mb));
    L.err = take(4 * sizeof(int));
    L.total = off;
    return L;
}
}  // namespace

extern "C" int smx_spd_inverse_seed_workspace_size(int64_t m, size_t *bytes) {
    if (m < 1 || m > 46340 || !bytes) return set_error(SMX_ERR_ARGUMENT, "smx_spd_inverse_seed_workspace_size: bad argument");
    *bytes = seed_layout(m).total;
    return SMX_OK;
}

extern "C" int smx_spd_inverse_seed(const double *G, int64_t m, double *X, void *workspace, size_t workspace_bytes,
                                    void *stream) {
    if (m < 1 || m > 46340 || !G || !X || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_spd_inverse_seed: bad argument");
    const SeedLayout L = seed_layout(m);
    if (workspace_bytes < L.total)
        return set_error(SMX_ERR_WORKSPACE, "smx_spd_inverse_seed: workspace %zu < %zu bytes", workspace_bytes, L.total);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *ws = (unsigned char *)workspace;
    SeedWorkspace w;
    w.a_slices = (__nv_bfloat16 *)(ws + L.a_sl);
    w.a_expo = (int32_t *)(ws + L.a_e);
    w.b_slices = (__nv_bfloat16 *)(ws + L.b_sl);
    w.b_expo = (int32_t *)(ws + L.b_e);
    w.T = (unsigned long long *)(ws + L.T);
    w.R = (float *)(ws + L.R);
    w.rowmax = (unsigned long long *)(ws + L.rowmax);
    w.gp = (float *)(ws + L.gp);
    w.gjws = (float *)(ws + L.gjws);
    w.base = (double *)(ws + L.base);
    w.err = (int *)(ws + L.err);
    w.flag = w.err + 1;
    SMX_TRY_CUDA(cudaMemsetAsync(w.T, 0, (size_t)m * m * sizeof(unsigned long long), s));
    SMX_TRY_CUDA(cudaMemsetAsync(w.R, 0, (size_t)m * m * sizeof(float), s));
    SMX_TRY_CUDA(cudaMemsetAsync(w.err, 0, 4 * sizeof(int), s));
    SMX_TRY_CUDA(cudaMemcpyAsync(X, G, (size_t)m * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
    int st = spd_inverse_seed(X, m, m, (double *)(ws + L.scratch), w, s);
    if (st) return st;
    int herr[2] = {0, 0};
    SMX_TRY_CUDA(cudaMemcpyAsync(herr, w.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (herr[0]) return set_error(SMX_ERR_CUDA, "smx_spd_inverse_seed: product kernel gave up waiting (code %d)", herr[0]);
    if (herr[1]) return set_error(SMX_ERR_NUMERIC, "smx_spd_inverse_seed: a pivot was not positive");
    return SMX_OK;
}
