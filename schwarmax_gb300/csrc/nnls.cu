// ADMM non-negative least squares for many right-hand sides
// (solve_nnls_admm_bootstrap, nnls.py:68-166; solve_nnls_admm, nnls.py:6-66).
//
// The reference factorises the n x n matrix Q + rho I = U^T U + (lambda/n + rho) I.
// The design matrix has fewer rows than columns (m < n), so the same inverse
// is applied through the Woodbury identity with the m x m matrix
//   G = c I + U U^T,   c = rho + lambda/n,   rho = (||U||_F^2 + lambda)/n,
// using (U^T U + c I)^-1 U^T = U^T G^-1.  With d = z - u the ADMM update
// w = (Q + rho I)^-1 (rho d + U^T y) is evaluated in residual form
//   w = k d + U^T G^-1 (y - k U d),   k = rho/c,
// which costs two skinny GEMMs with U and one application of G^-1 per
// iteration.  The mixed path forms H = G^-1 U once per solve and iterates
// w = D + H^T (y - U D): two skinny products per iteration (U D and H^T E).  The grouping matters in low precision: the algebraically equal
// k (d - U^T G^-1 U d) + U^T G^-1 y subtracts two vectors of the size of d whose
// difference is up to cond(G) times smaller, so rounding errors of G^-1 and of
// the products grow by cond(G) (about 1.8e3 at 16384 orbits); in residual form
// they only scale the correction U^T G^-1 r.  Then w^ = 1.6 w - 0.6 z,
// z = max(0, w^ + u), u = u + w^ - z exactly as nnls.py:151-158.  The kernels keep
// D = k (z - u), so that w = D + U^T G^-1 (y - U D).
//
// SMX_NNLS_FP64: every step in double (cuBLAS DSYRK/DGEMM, cuSOLVER DPOTRF/DPOTRS).
// SMX_NNLS_MIXED: U in float; every product on the bf16 tensor cores with
// FP64-grade accuracy by Ozaki splitting (split_gemm.cuh): U in 4 slices (31 bits
// below each row's or column's largest magnitude), the iterates' vectors in 5
// (39 bits), G^-1 in 5, H = G^-1 U in 4.  G = U U^T + cI is formed from the slices
// of U; G^-1 starts from a seed by Schur-complement recursion on split products
// (spd_inverse.cu, residual ~4e-5) and is refined by a Newton-Schulz step whose
// residual product uses 7 slices; the iterates z, u, D stay in double.
// At 16384 orbits (cond(G) = 1.8e3) the weights move the chi^2 by about 0.02
// when U is rounded to float, by about 40 when G^-1 is stored in float and by
// about 500 when the iterations run in float arithmetic, which is why the
// products are split rather than rounded.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cstdio>
#include <cmath>
#include <cstring>
#include <vector>

#include "smx_internal.cuh"
#include "split_gemm.cuh"

namespace smx {

// FP32 SPD inverse by blocked Gauss-Jordan (spd_inverse.cu)
int64_t spd_inverse_padded(int64_t m);
size_t spd_inverse_workspace(int64_t m);

struct Handles {
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    int device = -1;
};

static thread_local Handles g_handles;

static int get_handles(cudaStream_t s, Handles **out) {
    int dev = 0;
    SMX_TRY_CUDA(cudaGetDevice(&dev));
    Handles &h = g_handles;
    if (h.device != dev) {
        if (h.blas) cublasDestroy(h.blas);
        if (h.solver) cusolverDnDestroy(h.solver);
        h.blas = nullptr;
        h.solver = nullptr;
        if (cublasCreate(&h.blas) != CUBLAS_STATUS_SUCCESS) return set_error(SMX_ERR_CUDA, "cublasCreate failed");
        if (cusolverDnCreate(&h.solver) != CUSOLVER_STATUS_SUCCESS)
            return set_error(SMX_ERR_CUDA, "cusolverDnCreate failed");
        h.device = dev;
    }
    cublasSetStream(h.blas, s);
    cusolverDnSetStream(h.solver, s);
    *out = &h;
    return SMX_OK;
}

#define SMX_TRY_BLAS(expr)                                                                   \
    do {                                                                                     \
        cublasStatus_t _s = (expr);                                                          \
        if (_s != CUBLAS_STATUS_SUCCESS) return set_error(SMX_ERR_CUDA, "%s: cuBLAS status %d", #expr, (int)_s); \
    } while (0)
#define SMX_TRY_SOLVER(expr)                                                                 \
    do {                                                                                     \
        cusolverStatus_t _s = (expr);                                                        \
        if (_s != CUSOLVER_STATUS_SUCCESS) return set_error(SMX_ERR_CUDA, "%s: cuSOLVER status %d", #expr, (int)_s); \
    } while (0)

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// sliced operands of the split path (tile geometry only; pointers are set in run)
struct SplitShapes {
    split::Operand Ua, Ut, Xg, Ds, Es, Fs;   // Xg: G^-1 for the iterations
    split::Operand G7, X7, X4, R4;           // Newton-Schulz operands
};

static SplitShapes split_shapes(const smx_nnls_problem *p) {
    SplitShapes sh;
    const int64_t m = p->m, n = p->n, B = p->n_rhs;
    const int vt = 112;   // vector tiles: 112 right-hand sides per tile
    sh.Ua = split::make_operand(m, n, split::MT, 4);    // rows of U over orbits
    sh.Ut = split::make_operand(n, m, split::MT, 4);    // orbits over rows of U
    sh.Xg = split::make_operand(m, m, split::MT, 5);
    sh.Ds = split::make_operand(B, n, vt, 5);
    sh.Es = split::make_operand(B, m, vt, 5);   // jackknife: inputs of the Neumann terms
    sh.Fs = split::make_operand(B, m, vt, 5);
    sh.G7 = split::make_operand(m, m, split::MT, 7);
    sh.X7 = split::make_operand(m, m, 96, 7);
    sh.X4 = split::make_operand(m, m, split::MT, 4);
    sh.R4 = split::make_operand(m, m, split::MT, 4);
    return sh;
}

struct Layout {
    size_t U, G, work, info, frob, Z, Uu, D, E, F, Gt, total;
    // split path
    size_t Tacc, Racc, rowmax, err;
    size_t Ua, Ua_e, Ut, Ut_e, Xg, Xg_e, Ds, Ds_e, Es, Es_e, Fs, Fs_e;
    size_t G7, G7_e, X7, X7_e, X4, X4_e, R4, R4_e, Gf, gjws, seedbase, nsflag, Xd, Rd, Ebuf, Fbuf, gdiag, colmax;
    int lwork_s;   // float Cholesky / inverse scratch (floats)
    int64_t acc_elems;
    size_t work_bytes, host_bytes;   // device / host scratch of the factorisation and inversion
    int lwork;
};

// with_h: the bootstrap solver's accumulators also hold the m x n product O U that
// forms H = G^-1 U once per solve (the jackknife applies its own inverses and does not)
static int layout(const smx_nnls_problem *p, Layout *L, cusolverDnHandle_t solver, bool with_h = true) {
    const size_t m = p->m, n = p->n, B = p->n_rhs;
    const bool mixed = p->mode == SMX_NNLS_MIXED;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
    *L = Layout();
    L->U = take(m * n * sizeof(double));   // U = library x row scale in double for both modes
    L->G = take(m * m * sizeof(double));
    int lwork = 0, lw_f = 0, lw_i = 0;
    if (solver) {
        if (!mixed) {
            SMX_TRY_SOLVER(cusolverDnDpotrf_bufferSize(solver, CUBLAS_FILL_MODE_LOWER, (int)m, nullptr, (int)m, &lwork));
        }
    } else {
        lwork = lw_f = lw_i = (int)(m * 256 + (1 << 20));   // generous estimate for size queries without a handle
    }
    L->lwork = lwork;
    L->lwork_s = lw_f > lw_i ? lw_f : lw_i;
    L->work_bytes = mixed ? 256 : (size_t)lwork * sizeof(double);
    L->host_bytes = 0;
    L->work = take(L->work_bytes);
    L->info = take(sizeof(int) * 4);
    L->frob = take(sizeof(double) * 4);   // ||U||_F^2, k (double), k (float)
    L->Z = take(n * B * sizeof(double));
    L->Uu = take(n * B * sizeof(double));
    L->D = take(n * B * sizeof(double));
    if (!mixed) {
        L->E = take(m * B * sizeof(double));
        L->Gt = take(n * B * sizeof(double));
    } else {
        const SplitShapes sh = split_shapes(p);
        const size_t mx = m > n ? m : n;
        L->acc_elems = (int64_t)(m * m > mx * B ? m * m : mx * B);
        if (with_h && (int64_t)(m * n) > L->acc_elems) L->acc_elems = (int64_t)(m * n);
        L->Tacc = take(L->acc_elems * sizeof(unsigned long long));
        L->Racc = take(L->acc_elems * sizeof(float));
        L->rowmax = take(mx * sizeof(unsigned long long));
        L->err = take(sizeof(int) * 4);
        auto op = [&](const split::Operand &o, size_t &sl, size_t &ex) {
            sl = take(o.slice_bytes());
            ex = take((size_t)o.row_tiles * o.tile_rows * sizeof(int32_t));
        };
        op(sh.Ua, L->Ua, L->Ua_e);
        op(sh.Ut, L->Ut, L->Ut_e);
        op(sh.Xg, L->Xg, L->Xg_e);
        op(sh.Ds, L->Ds, L->Ds_e);
        op(sh.Es, L->Es, L->Es_e);
        op(sh.Fs, L->Fs, L->Fs_e);
        op(sh.G7, L->G7, L->G7_e);
        op(sh.X7, L->X7, L->X7_e);
        op(sh.X4, L->X4, L->X4_e);
        op(sh.R4, L->R4, L->R4_e);
        // the seed's Gauss-Jordan blocks (at most kSeedBaseRows rows)
        const int64_t mb = (int64_t)m < kSeedBaseRows ? (int64_t)m : kSeedBaseRows;
        const int64_t mp = spd_inverse_padded(mb);
        L->Gf = take((size_t)mp * mp * sizeof(float));
        L->gjws = take(spd_inverse_workspace(mb));
        L->seedbase = take((size_t)2 * mb * mb * sizeof(double));
        L->nsflag = take(16 * sizeof(int));
        L->Xd = take(m * m * sizeof(double));
        L->Rd = take(m * m * sizeof(double));
        L->Ebuf = take(m * B * sizeof(double));
        L->Fbuf = take(m * B * sizeof(double));
        L->gdiag = take(m * sizeof(double));
        L->colmax = take(3 * B * sizeof(unsigned long long));
    }
    L->total = off;
    return SMX_OK;
}

// U[i*m + r] = lib[i*ld + row_map[r]] * row_scale[r]; a row index outside
// [0, ld) is not read: the entry is set to 0 and flag[0] records the error.
template <typename TL, typename TU>
__global__ void build_u_kernel(const TL *__restrict__ lib, int64_t ld, const int32_t *__restrict__ row_map,
                               const double *__restrict__ row_scale, int64_t m, int64_t n, TU *U, int *flag) {
    for (int64_t i = blockIdx.y; i < n; i += gridDim.y) {
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
            const int64_t src = row_map[r];
            if (src < 0 || src >= ld) {
                flag[0] = 1;
                U[i * m + r] = TU(0);
            } else {
                U[i * m + r] = TU((double)lib[i * ld + src] * row_scale[r]);
            }
        }
    }
}

template <typename TU>
__global__ void frob_kernel(const TU *__restrict__ U, int64_t count, double *out) {
    double s = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        const double v = (double)U[k];
        s += v * v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(out, s);
    }
}

__global__ void add_diag_kernel(double *G, int64_t m, const double *frob, double lambda, double n) {
    const double c = (frob[0] + lambda) / n + lambda / n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        G[i * m + i] += c;
}

template <typename T>
__global__ void admm_init_kernel(T *Z, T *Uu, T *D, int64_t count, double w_init, const double *coefp) {
    const T w = T(w_init), dk = T(coefp[0] * w_init);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        Z[k] = w;
        Uu[k] = T(0);
        D[k] = dk;
    }
}

// coef[0] = k = rho / (rho + lambda/n) with rho = (||U||_F^2 + lambda)/n, in double and float
__global__ void admm_coef_kernel(const double *frob, double lambda, double n, double *coef) {
    const double rho = (frob[0] + lambda) / n;
    coef[0] = rho / (rho + lambda / n);
    ((float *)(coef + 1))[0] = (float)coef[0];
}

// w = D + U^T G^-1 (y - U D);  w^ = 1.6 w - 0.6 z;  z = max(0, w^ + u);  u += w^ - z;  D = k (z - u)
template <typename T>
__global__ void admm_update_kernel(const T *__restrict__ Gt, T *Z, T *Uu, T *D, int64_t count, const double *coefp) {
    const T coef = sizeof(T) == 8 ? T(coefp[0]) : T(((const float *)(coefp + 1))[0]);
    const T alpha = T(1.6);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        const T z = Z[k], u = Uu[k];
        const T w = D[k] + Gt[k];
        const T wh = alpha * w + (T(1) - alpha) * z;
        T zn = wh + u;
        zn = zn > T(0) ? zn : T(0);
        const T un = u + wh - zn;
        Z[k] = zn;
        Uu[k] = un;
        D[k] = coef * (zn - un);
    }
}

static inline unsigned grid1d(int64_t count, int bs = 256) {
    int64_t g = (count + bs - 1) / bs;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return (unsigned)g;
}

// ------------------------------------------------------------ split path

// exact power of two 2^p as a double, |p| < 1022
__device__ __forceinline__ double pow2(int p) { return __longlong_as_double((long long)(1023 + p) << 52); }

// value of a split product: 2^(eA_r + eB_j - 14) (T 2^-t_shift + R), t_shift = 8 (exact levels - 1)
__device__ __forceinline__ double product_of(long long t, float r, int ea, int eb, int t_shift) {
    const double v = (double)t * pow2(-t_shift) + (double)r;
    return v * pow2(ea + eb - 14);
}
__device__ __forceinline__ double product_value(const unsigned long long *T, const float *R, int64_t idx, int ea,
                                                int eb, int t_shift = 16) {
    return product_of((long long)T[idx], R[idx], ea, eb, t_shift);
}

enum { COL_INIT = 0, COL_RESID = 1, COL_PLAIN = 2, COL_UPDATE = 3 };

constexpr int kNsMaxSteps = 5;   // Newton-Schulz steps at most (a seed residual of 0.2 needs 4)
constexpr double kNsStopResidual2 = 1e-8;   // ||R||_F^2 of the input of the last step
// Slice pairs s + t <= 7 of the residual G X (7 x 7 slices).  5 x 5 slices with pairs
// s + t <= 6 saved 4 ms per config-1 solve but moved the largest bootstrap delta chi^2
// against FP64 from 1.8e-3 to 1.5e-2 (the residual's error enters G^-1 directly).
constexpr int kNsResidualLevels = 7;
constexpr int kNsUpdateLevels = 5;     // slice pairs s + t <= 5 of the update X R (4 x 4 slices)

constexpr int VS = 5;          // slices of the vector operands: 39 bits below each column's largest magnitude
// Slice pairs (s, t) of the skinny products U D and H^T E with s + t <= kSkinnyLevels.
// The pairs left out (s + t >= 6) weigh 2^-32 of max|A| max|B| per term, the size of
// the 31-bit slicing of U and H; at 16,384 orbits x 6,608 rows x 100 right-hand sides
// levels 7, 6 and 5 gave a largest bootstrap delta chi^2 against FP64 of 1.3e-3, 1.3e-3
// and 1.5e-3 on the same library; at level 5 the products form 10 slice pairs instead of 17.
constexpr int kSkinnyLevels = 5;
constexpr int COL_CHUNK = 1024;   // k per CTA of the column kernels

struct ColArgs {
    int64_t K, n_rhs;
    unsigned long long *T;   // product of the previous step (K x n_rhs, ld K), zeroed here after use
    float *R;
    const int32_t *eA;       // its row exponents (K) and column exponents (n_rhs)
    const int32_t *eB;
    const double *Y;         // COL_RESID: Y[j K + k]
    double *E;               // COL_RESID writes E, COL_PLAIN reads it (K x n_rhs)
    const double *g;         // COL_PLAIN: diagonal of G^-1, applied exactly
    double *Z, *Uu, *D;      // COL_INIT / COL_UPDATE: iterates (K x n_rhs)
    double *V;               // the column values to slice (E, F or D)
    unsigned long long *colmax;    // max |V| of each column, as ordered bits
    unsigned long long *reset;     // column maxima of another operand, cleared here (n_rhs)
    const double *coefp;
    const double *colcoef;   // optional per-column k (the jackknife's replicates), else coefp[0]
    double w_init;
    __nv_bfloat16 *slices;   // output operand: n_rhs x K, VS slices, tiles of tile_rows x KT
    int32_t *expo;
    int64_t k_tiles, slice_elems;
    int tile_rows;
    int t_shift;             // units of the product's T: 2^-t_shift
    // COL_UPDATE of the jackknife (optional): w -= sum_q cvec[j, q] hrows[j, q, :]
    const double *hrows, *cvec;
    int max_drop;
};

// Phase 1 of a column step, grid (K / COL_CHUNK, n_rhs): forms the new column values
// and their largest magnitude per column.
//   COL_INIT:   z = w_init, u = 0, D = k w_init
//   COL_RESID:  E = Y - U D                 (the residual y - U D)
//   COL_PLAIN:  F = g E + O E               (G^-1 = diag(g) + O; O E is the product)
//   COL_UPDATE: w = D + U^T F; w^ = 1.6 w - 0.6 z; z = max(0, w^ + u); u += w^ - z; D = k (z - u)
template <int MODE>
__global__ void __launch_bounds__(256) column_values_kernel(const ColArgs a) {
    constexpr int PER = COL_CHUNK / 256;   // values per thread
    const int64_t j = blockIdx.y, K = a.K;
    if (blockIdx.x == 0 && blockIdx.y == 0)
        for (int i = threadIdx.x; i < a.n_rhs; i += blockDim.x) a.reset[i] = 0ull;
    const int eb = (MODE == COL_INIT) ? 0 : a.eB[j];
    const double coef = a.colcoef ? a.colcoef[j] : a.coefp[0];
    const int64_t kb = blockIdx.x * (int64_t)COL_CHUNK;
    const int64_t k1 = kb + COL_CHUNK < K ? kb + COL_CHUNK : K;
    // every load of the thread's PER values is issued before any store, so that
    // their latencies overlap (one value after another, each waited on its loads)
    long long t[PER];
    float r[PER];
    int ea[PER];
    double x[PER], y[PER], uu[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int64_t k = kb + threadIdx.x + q * 256, idx = k + K * j;
        if (k >= k1) continue;
        if (MODE != COL_INIT) {
            t[q] = (long long)a.T[idx];
            r[q] = a.R[idx];
            ea[q] = a.eA[k];
        }
        if (MODE == COL_UPDATE) {
            x[q] = a.D[idx];
            y[q] = a.Z[idx];
            uu[q] = a.Uu[idx];
        } else if (MODE == COL_RESID) {
            x[q] = a.Y[idx];
        } else if (MODE == COL_PLAIN) {
            x[q] = a.E[idx];
            y[q] = a.g[k];
        }
    }
    double mx = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int64_t k = kb + threadIdx.x + q * 256, idx = k + K * j;
        if (k >= k1) continue;
        double v;
        if (MODE == COL_INIT) {
            a.Z[idx] = a.w_init;
            a.Uu[idx] = 0.0;
            v = coef * a.w_init;
            a.D[idx] = v;
        } else {
            const double pv = product_of(t[q], r[q], ea[q], eb, a.t_shift);
            a.T[idx] = 0ull;
            a.R[idx] = 0.0f;
            if (MODE == COL_UPDATE) {
                const double z = y[q], u = uu[q];
                double w = x[q] + pv;
                if (a.hrows)
                    for (int t = 0; t < a.max_drop; ++t)
                        w -= a.cvec[j * a.max_drop + t] * a.hrows[(j * a.max_drop + t) * K + k];
                const double wh = 1.6 * w - 0.6 * z;
                double zn = wh + u;
                zn = zn > 0.0 ? zn : 0.0;
                const double un = u + wh - zn;
                a.Z[idx] = zn;
                a.Uu[idx] = un;
                v = coef * (zn - un);
                a.D[idx] = v;
            } else if (MODE == COL_RESID) {
                v = x[q] - pv;
                a.E[idx] = v;
            } else {
                v = pv;
                v += y[q] * x[q];
                a.V[idx] = v;
            }
        }
        mx = fmax(mx, fabs(v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m2 = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m2 = fmax(m2, red[w]);
        atomicMax(a.colmax + j, (unsigned long long)__double_as_longlong(m2));
    }
}

// Phase 2, grid (K / COL_CHUNK, n_rhs), COL_CHUNK / 8 threads: the column's scale
// 2^e > max |V| and the VS slices of every value, written as 16-byte vectors into
// the B-operand tiles of the next product (padding k stays zero).
__global__ void __launch_bounds__(COL_CHUNK / 8) column_slices_kernel(const ColArgs a) {
    const int64_t j = blockIdx.y, K = a.K;
    const double mx = __longlong_as_double((long long)a.colmax[j]);
    int e = 0;
    if (mx > 0) frexp(mx, &e);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.expo[j] = e;
    const int64_t jt = j / a.tile_rows, jr = j % a.tile_rows;
    const int64_t g = (blockIdx.x * (int64_t)COL_CHUNK) / 8 + threadIdx.x;   // group of 8 k
    if (g >= a.k_tiles * (split::KT / 8)) return;
    __align__(16) __nv_bfloat16 sl[VS][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int64_t k = g * 8 + q;
        const double v = k < K ? a.V[k + K * j] : 0.0;
        __nv_bfloat16 d[VS];
        split::make_slices<VS>(v, e, d);
#pragma unroll
        for (int s = 0; s < VS; ++s) sl[s][q] = d[s];
    }
    const int64_t k0 = g * 8, kt = k0 / split::KT;
    const int64_t base = (jt * a.k_tiles + kt) * (int64_t)a.tile_rows * split::KT +
                         split::tile_offset((int)jr, (int)(k0 % split::KT), a.tile_rows);
#pragma unroll
    for (int s = 0; s < VS; ++s) *(uint4 *)(a.slices + s * a.slice_elems + base) = *(const uint4 *)sl[s];
}

// Gram combine: G = 2^(e_r + e_c - 14)(T/256 + R) + c I from the lower-triangle
// product tiles, written to both triangles in double and to a float copy for the
// seed factorisation; T and R are cleared for the next product.
__global__ void gram_combine_kernel(unsigned long long *T, float *R, const int32_t *e, double *G, int64_t m,
                                    const double *frob, double lambda, double n) {
    const double c = (frob[0] + lambda) / n + lambda / n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * m; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k % m, col = k / m;
        if (r >= col) {
            double v = product_value(T, R, k, e[r], e[col]);
            if (r == col) v += c;
            G[k] = v;
            G[col + m * r] = v;
        }
        T[k] = 0ull;
        R[k] = 0.0f;
    }
}

// Newton-Schulz seed: X0 = the symmetric part of the float inverse (padded, leading
// dimension mp), in double
// Device-side control of the Newton-Schulz steps (no host read-back): flag[0] = 1
// while steps are still to run; after the residual of a step, with ss = ||I - G X||_F^2
// of the step's input: a step whose input is below thr2 is the last one; an input at
// or above 1/4 (not converging) stops the iteration with flag[1] = 1; flag[2] = 1
// once a step with a converged input has run.  skip = flag[3] = !flag[0] for the
// kernels of the next step.
__global__ void ns_gate_kernel(const double *rss, double thr2, int *flag) {
    if (!flag[0]) return;
    const double ss = rss[0];
    if (!(ss < 0.25)) {
        flag[0] = 0;
        flag[1] = 1;
    } else if (ss <= thr2) {
        flag[0] = 0;
        flag[2] = 1;
    }
}
__global__ void ns_skip_kernel(int *flag) { flag[3] = flag[0] ? 0 : 1; }
__global__ void ns_init_kernel(int *flag) {
    flag[0] = 1;
    flag[1] = 0;
    flag[2] = 0;
    flag[3] = 0;
}
// final verdict of the set-up: dinfo[1] = 1 when the inverse did not converge
__global__ void ns_verdict_kernel(const int *flag, int *dinfo) {
    if (flag[1] || !flag[2]) dinfo[1] = 1;
}

// residual R = I - G X of a Newton-Schulz step.  G and X are dominated by their
// diagonals, so G X = D_G X + O_G D_X + O_G O_X with D the diagonals and O the
// rest: the first two terms are formed here in double, only O_G O_X comes from
// the split product (T in units of 2^-t_shift).  rss receives sum R_ij^2
// (||R||_F^2, a bound on ||R||_2^2).
__global__ void ns_residual_kernel(unsigned long long *T, float *Racc, const int32_t *eG, const int32_t *eX,
                                   const double *G, const double *X, double *Rd, int64_t m, double *rss,
                                   const int *skip, int t_shift) {
    if (*skip) return;
    double acc = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * m; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k % m, col = k / m;
        double gx = product_of((long long)T[k], Racc[k], eG[r], eX[col], t_shift);
        gx += G[r + m * r] * X[k];
        if (r != col) gx += G[k] * X[col + m * col];
        const double v = (r == col ? 1.0 : 0.0) - gx;
        Rd[k] = v;
        acc += v * v;
        T[k] = 0ull;
        Racc[k] = 0.0f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(rss, acc);
}

// X <- X + X R.  X R = X - X G X is symmetric, so the product is formed on the lower
// tiles only (tiles of split::MT rows) and every element above the diagonal takes the
// value of its mirror; X stays exactly symmetric.  T and R are cleared by a separate
// pass (a thread may read the mirror of an element another thread is done with).
__global__ void ns_update_kernel(const unsigned long long *T, const float *Racc, const int32_t *eX,
                                 const int32_t *eR, double *X, int64_t m, const int *skip, int t_shift) {
    if (*skip) return;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * m; k += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = k % m, j = k / m;
        if (j > i) {   // (j, i) lies in a lower tile
            const int64_t t = i;
            i = j;
            j = t;
        }
        X[k] += product_value(T, Racc, i + m * j, eX[i], eR[j], t_shift);
    }
}

// G^-1 = diag(g) + O: the diagonal dominates its rows (about 14x the largest
// off-diagonal entry at 16384 orbits), so it is applied exactly in double and
// only O goes through the split product, whose row scales then follow O.
__global__ void split_diag_kernel(double *X, double *g, int64_t m) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        g[r] = X[r + m * r];
        X[r + m * r] = 0.0;
    }
}

__global__ void clear_kernel(unsigned long long *T, float *R, int64_t count) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        T[k] = 0ull;
        R[k] = 0.0f;
    }
}

// H = G^-1 U = diag(g) U + O U in place of U (both m x n column-major): the product
// O U arrives as T, R with row exponents of O and column exponents of U; T, R cleared.
__global__ void h_combine_kernel(unsigned long long *T, float *R, const int32_t *eO, const int32_t *eU,
                                 const double *g, double *U, int64_t m, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k % m, i = k / m;
        U[k] = g[r] * U[k] + product_value(T, R, k, eO[r], eU[i]);
        T[k] = 0ull;
        R[k] = 0.0f;
    }
}

__global__ void rownorm_kernel(const double *__restrict__ U, int64_t m, int64_t n, double *out);

// The set-up of the mixed path shared by the bootstrap and jackknife solvers: U in
// double, ||U||_F^2 and the ADMM coefficient, U sliced both ways, G = U U^T + c I
// from the slices, G^-1 by a float seed and Newton-Schulz steps, and G^-1 split into
// its diagonal (gdiag) and the sliced off-diagonal part (sh.Xg; Xd keeps it in double).
struct MixedState {
    SplitShapes sh;
    unsigned long long *Tacc, *rowmax;
    float *Racc;
    int *derr;
    double *U, *Xd, *gdiag;
};

template <typename TL>
static int mixed_setup(const smx_nnls_problem *p, const TL *lib, const int32_t *row_map, const double *row_scale,
                       unsigned char *ws, const Layout &L, Handles *h, cudaStream_t s, MixedState &S,
                       bool make_h = false, double *rownorm = nullptr) {
    const int64_t m = p->m, n = p->n;
    const double lam = p->lambda_reg;
    double *G = (double *)(ws + L.G);
    double *frob = (double *)(ws + L.frob);
    int *dinfo = (int *)(ws + L.info);
    dim3 gb((unsigned)((m + 255) / 256 < 65535 ? (m + 255) / 256 : 65535), (unsigned)(n < 65535 ? n : 65535));
    // U in double: rounding library x row scale to float (2^-24 of every entry, and
    // |U|_F^2 and rho with it) moved the bootstrap chi^2 by up to 0.1 at config 1;
    // the slices below keep 31 bits of each row's largest entry
    double *U = (double *)(ws + L.U);
    build_u_kernel<TL, double><<<gb, 256, 0, s>>>(lib, p->ld_lib, row_map, row_scale, m, n, U, dinfo + 3);
    count_launch();
    frob_kernel<double><<<grid1d(m * n), 256, 0, s>>>(U, m * n, frob);
    count_launch();
    admm_coef_kernel<<<1, 1, 0, s>>>(frob, lam, (double)n, frob + 1);
    count_launch();
    if (rownorm) {   // ||U_r||^2 of every design row, before U is replaced by H
        SMX_TRY_CUDA(cudaMemsetAsync(rownorm, 0, m * sizeof(double), s));
        rownorm_kernel<<<dim3((unsigned)((m + 255) / 256), 64), 256, 0, s>>>(U, m, n, rownorm);
        count_launch();
    }
    SplitShapes sh = split_shapes(p);
    sh.Ua.slices = (__nv_bfloat16 *)(ws + L.Ua);
    sh.Ua.expo = (int32_t *)(ws + L.Ua_e);
    sh.Ut.slices = (__nv_bfloat16 *)(ws + L.Ut);
    sh.Ut.expo = (int32_t *)(ws + L.Ut_e);
    sh.Xg.slices = (__nv_bfloat16 *)(ws + L.Xg);
    sh.Xg.expo = (int32_t *)(ws + L.Xg_e);
    sh.Ds.slices = (__nv_bfloat16 *)(ws + L.Ds);
    sh.Ds.expo = (int32_t *)(ws + L.Ds_e);
    sh.Es.slices = (__nv_bfloat16 *)(ws + L.Es);
    sh.Es.expo = (int32_t *)(ws + L.Es_e);
    sh.Fs.slices = (__nv_bfloat16 *)(ws + L.Fs);
    sh.Fs.expo = (int32_t *)(ws + L.Fs_e);
    sh.G7.slices = (__nv_bfloat16 *)(ws + L.G7);
    sh.G7.expo = (int32_t *)(ws + L.G7_e);
    sh.X7.slices = (__nv_bfloat16 *)(ws + L.X7);
    sh.X7.expo = (int32_t *)(ws + L.X7_e);
    sh.X4.slices = (__nv_bfloat16 *)(ws + L.X4);
    sh.X4.expo = (int32_t *)(ws + L.X4_e);
    sh.R4.slices = (__nv_bfloat16 *)(ws + L.R4);
    sh.R4.expo = (int32_t *)(ws + L.R4_e);
    unsigned long long *Tacc = (unsigned long long *)(ws + L.Tacc);
    float *Racc = (float *)(ws + L.Racc);
    unsigned long long *rowmax = (unsigned long long *)(ws + L.rowmax);
    int *derr = (int *)(ws + L.err);
    SMX_TRY_CUDA(cudaMemsetAsync(derr, 0, 4 * sizeof(int), s));
    clear_kernel<<<grid1d(L.acc_elems), 256, 0, s>>>(Tacc, Racc, L.acc_elems);
    count_launch();
    // the vector operands' padding (right-hand sides beyond n_rhs) stays zero
    SMX_TRY_CUDA(cudaMemsetAsync(sh.Ds.slices, 0, sh.Ds.slice_bytes(), s));
    SMX_TRY_CUDA(cudaMemsetAsync(sh.Es.slices, 0, sh.Es.slice_bytes(), s));
    SMX_TRY_CUDA(cudaMemsetAsync(sh.Fs.slices, 0, sh.Fs.slice_bytes(), s));
    int st;
    // U split both ways: rows of U over orbits (U D, U U^T) and orbits over rows (U^T F)
    if ((st = split::slice_rows<double>(U, 1, m, sh.Ua, rowmax, s))) return st;
    if ((st = split::slice_rows<double>(U, m, 1, sh.Ut, rowmax, s))) return st;
    // G = U U^T + c I from the sliced U (31 bits below each row's largest entry), all slice pairs
    split::Acc acc{Tacc, Racc, m};
    float *Gp = (float *)(ws + L.Gf);
    double *Xd = (double *)(ws + L.Xd), *Rd = (double *)(ws + L.Rd);
    if ((st = split::gemm(sh.Ua, sh.Ua, acc, true, derr, s))) return st;
    gram_combine_kernel<<<grid1d(m * m), 256, 0, s>>>(Tacc, Racc, sh.Ua.expo, G, m, frob, lam, (double)n);
    count_launch();
    // G^-1: a seed of FP32 quality (Schur-complement recursion on split products with
    // FP32 Gauss-Jordan blocks, spd_inverse_seed), then Newton-Schulz steps
    //   R = I - G X (diagonals exact, off-diagonal parts as a 7 x 7 split
    //   product), X <- X + X R.
    // The new X has residual R^2, whose 2-norm is at most ||R||_F^2: steps
    // continue until a step's input has ||R||_F <= 1e-4, so the result has
    // ||I - G X|| <= 1e-8 and X a relative error of at most 1e-8, far below the
    // 2^-31 slicing of U and H in every iteration (a seed with ||R||_F ~ 5e-3 needs
    // two steps: 5e-3 -> 3e-5 -> 1e-9).
    // The stopping rule runs on the device (ns_gate_kernel): the kernels of a step
    // that is not needed return at once, and nothing is read back here.
    int *nsf = (int *)(ws + L.nsflag);
    {
        // the slice buffers of the Newton-Schulz operands, the accumulators and Rd are
        // free until the first step
        SeedWorkspace sw;
        sw.a_slices = sh.G7.slices;
        sw.a_expo = sh.G7.expo;
        sw.b_slices = sh.X7.slices;
        sw.b_expo = sh.X7.expo;
        sw.T = Tacc;
        sw.R = Racc;
        sw.rowmax = rowmax;
        sw.gp = Gp;
        sw.gjws = (float *)(ws + L.gjws);
        sw.base = (double *)(ws + L.seedbase);
        sw.err = derr;
        sw.flag = dinfo + 1;
        SMX_TRY_CUDA(cudaMemcpyAsync(Xd, G, (size_t)m * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if ((st = spd_inverse_seed(Xd, m, m, Rd, sw, s))) return st;
    }
    if ((st = split::slice_rows<double>(G, 1, m, sh.G7, rowmax, s, true))) return st;   // O_G
    double *rss = frob + 3;
    ns_init_kernel<<<1, 1, 0, s>>>(nsf);
    count_launch();
    const int *skip = nsf + 3;
    for (int step = 0; step < kNsMaxSteps; ++step) {
        // Residual products keep 7 slices in every step (a first step with 3-slice products,
        // whose output only needs to be as good as ||R0||^2 ~ 4e-6, left a residual too
        // large for the second step to be the last, and so cost a third step), with the
        // slice pairs s + t <= 7: the pairs left out weigh 2^-48 of max|O_G| max|O_X| per
        // term.  The update X R only has to be good to a fraction of ||R|| <= 2e-3 of X:
        // 4 slices and pairs s + t <= 5 (2^-32 per term).
        const split::Operand &g = sh.G7, &x = sh.X7, &xr = sh.X4, &rr = sh.R4;
        if ((st = split::slice_rows<double>(Xd, m, 1, sh.X7, rowmax, s, true, skip))) return st;   // O_X columns over k
        if ((st = split::gemm(g, x, acc, false, derr, s, kNsResidualLevels, skip))) return st;
        SMX_TRY_CUDA(cudaMemsetAsync(rss, 0, sizeof(double), s));
        ns_residual_kernel<<<grid1d(m * m), 256, 0, s>>>(Tacc, Racc, sh.G7.expo, sh.X7.expo, G, Xd, Rd, m, rss, skip,
                                                         8 * (split::exact_levels(g, x) - 1));
        ns_gate_kernel<<<1, 1, 0, s>>>(rss, kNsStopResidual2, nsf);
        count_launch(2);
        if ((st = split::slice_rows<double>(Xd, 1, m, sh.X4, rowmax, s, false, skip))) return st;   // X rows over k
        if ((st = split::slice_rows<double>(Rd, m, 1, sh.R4, rowmax, s, false, skip))) return st;   // R columns over k
        if ((st = split::gemm(xr, rr, acc, true, derr, s, kNsUpdateLevels, skip))) return st;
        ns_update_kernel<<<grid1d(m * m), 256, 0, s>>>(Tacc, Racc, sh.X4.expo, sh.R4.expo, Xd, m, skip,
                                                       8 * (split::exact_levels(xr, rr) - 1));
        clear_kernel<<<grid1d(m * m), 256, 0, s>>>(Tacc, Racc, m * m);
        ns_skip_kernel<<<1, 1, 0, s>>>(nsf);
        count_launch(3);
    }
    ns_verdict_kernel<<<1, 1, 0, s>>>(nsf, dinfo);
    count_launch();
    double *gdiag = (double *)(ws + L.gdiag);
    split_diag_kernel<<<grid1d(m), 256, 0, s>>>(Xd, gdiag, m);
    count_launch();
    if ((st = split::slice_rows<double>(Xd, 1, m, sh.Xg, rowmax, s))) return st;   // O rows over columns
    if (make_h) {
        // H = G^-1 U, once per solve: every iteration then needs U D and H^T E only
        // (w = D + H^T (y - U D)), in place of U D, G^-1 E and U^T F.  U is overwritten
        // by H, and the slices of U^T (orbits over rows) by those of H^T.
        // pairs s + t <= 6: the pairs left out weigh 2^-40 of max|O| max|U| per term, far
        // below the 31-bit slicing of U and of H itself (4 slices of O with pairs
        // s + t <= 5 moved the largest bootstrap delta chi^2 at config 1 to 0.16)
        split::Acc acc_h{Tacc, Racc, m};
        if ((st = split::gemm(sh.Xg, sh.Ut, acc_h, false, derr, s, 6))) return st;   // O U
        h_combine_kernel<<<grid1d(m * n), 256, 0, s>>>(Tacc, Racc, sh.Xg.expo, sh.Ut.expo, gdiag, U, m, n);
        count_launch();
        if ((st = split::slice_rows<double>(U, m, 1, sh.Ut, rowmax, s))) return st;   // H^T: orbits over rows
    }
    S.sh = sh;
    S.Tacc = Tacc;
    S.Racc = Racc;
    S.rowmax = rowmax;
    S.derr = derr;
    S.U = U;
    S.Xd = Xd;
    S.gdiag = gdiag;
    return SMX_OK;
}

template <typename TL>
static int run(const smx_nnls_problem *p, const TL *lib, const int32_t *row_map, const double *row_scale,
               const double *Y, double *Z_out, unsigned char *ws, const Layout &L, Handles *h, cudaStream_t s) {
    const int64_t m = p->m, n = p->n, B = p->n_rhs;
    const bool mixed = p->mode == SMX_NNLS_MIXED;
    const double lam = p->lambda_reg;
    double *G = (double *)(ws + L.G);
    double *frob = (double *)(ws + L.frob);
    int *dinfo = (int *)(ws + L.info);
    SMX_TRY_CUDA(cudaMemsetAsync(frob, 0, sizeof(double), s));
    SMX_TRY_CUDA(cudaMemsetAsync(dinfo, 0, 4 * sizeof(int), s));
    dim3 gb((unsigned)((m + 255) / 256 < 65535 ? (m + 255) / 256 : 65535), (unsigned)(n < 65535 ? n : 65535));
    const double one = 1.0, zero = 0.0, mone = -1.0;
    std::vector<unsigned char> host_ws(L.host_bytes > 0 ? L.host_bytes : 1);   // outlives the final synchronize
    SMX_TRY_BLAS(cublasSetMathMode(h->blas, CUBLAS_DEFAULT_MATH));
    if (!mixed) {
        double *U = (double *)(ws + L.U);
        build_u_kernel<TL, double><<<gb, 256, 0, s>>>(lib, p->ld_lib, row_map, row_scale, m, n, U, dinfo + 3);
        count_launch();
        frob_kernel<double><<<grid1d(m * n), 256, 0, s>>>(U, m * n, frob);
        count_launch();
        admm_coef_kernel<<<1, 1, 0, s>>>(frob, lam, (double)n, frob + 1);
        count_launch();
        SMX_TRY_BLAS(cublasDsyrk(h->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, (int)m, (int)n, &one, U, (int)m, &zero,
                                 G, (int)m));
        add_diag_kernel<<<grid1d(m), 256, 0, s>>>(G, m, frob, lam, (double)n);
        count_launch();
        SMX_TRY_SOLVER(cusolverDnDpotrf(h->solver, CUBLAS_FILL_MODE_LOWER, (int)m, G, (int)m, (double *)(ws + L.work),
                                        L.lwork, dinfo));
        double *Z = (double *)(ws + L.Z), *Uu = (double *)(ws + L.Uu), *D = (double *)(ws + L.D),
               *E = (double *)(ws + L.E), *Gt = (double *)(ws + L.Gt);
        admm_init_kernel<double><<<grid1d(n * B), 256, 0, s>>>(Z, Uu, D, n * B, p->w_init, frob + 1);
        count_launch();
        for (int it = 0; it < p->maxiter; ++it) {
            // E = G^-1 (Y - U D)
            SMX_TRY_CUDA(cudaMemcpyAsync(E, Y, sizeof(double) * m * B, cudaMemcpyDeviceToDevice, s));
            SMX_TRY_BLAS(cublasDgemm(h->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, (int)B, (int)n, &mone, U, (int)m, D,
                                     (int)n, &one, E, (int)m));
            SMX_TRY_SOLVER(cusolverDnDpotrs(h->solver, CUBLAS_FILL_MODE_LOWER, (int)m, (int)B, G, (int)m, E, (int)m,
                                            dinfo + 2));
            SMX_TRY_BLAS(cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)B, (int)m, &one, U, (int)m, E,
                                     (int)m, &zero, Gt, (int)n));
            admm_update_kernel<double><<<grid1d(n * B), 256, 0, s>>>(Gt, Z, Uu, D, n * B, frob + 1);
            count_launch();
        }
        SMX_TRY_CUDA(cudaMemcpyAsync(Z_out, Z, sizeof(double) * n * B, cudaMemcpyDeviceToDevice, s));
    } else {
        MixedState S;
        int st;
        if ((st = mixed_setup<TL>(p, lib, row_map, row_scale, ws, L, h, s, S, true))) return st;
        SplitShapes &sh = S.sh;
        unsigned long long *Tacc = S.Tacc;
        float *Racc = S.Racc;
        int *derr = S.derr;
        double *gdiag = S.gdiag, *Ebuf = (double *)(ws + L.Ebuf);
        double *Z = (double *)(ws + L.Z), *Uu = (double *)(ws + L.Uu), *D = (double *)(ws + L.D);
        const double *coefp = frob + 1;
        // column maxima of the two vector operands (D, E), cleared once here and
        // afterwards by the phase-1 kernel of the operand that follows each one
        unsigned long long *cmD = (unsigned long long *)(ws + L.colmax), *cmE = cmD + B;
        SMX_TRY_CUDA(cudaMemsetAsync(cmD, 0, 3 * B * sizeof(unsigned long long), s));
        auto col = [&](int mode, int64_t K, const int32_t *eA, const int32_t *eB, split::Operand &out,
                       int t_shift) -> int {
            ColArgs a;
            memset(&a, 0, sizeof(a));
            a.K = K;
            a.n_rhs = B;
            a.T = Tacc;
            a.R = Racc;
            a.eA = eA;
            a.eB = eB;
            a.Y = Y;
            a.E = Ebuf;
            a.g = gdiag;
            a.Z = Z;
            a.Uu = Uu;
            a.D = D;
            a.coefp = coefp;
            a.colcoef = nullptr;
            a.w_init = p->w_init;
            a.slices = out.slices;
            a.expo = out.expo;
            a.k_tiles = out.k_tiles;
            a.slice_elems = out.slice_elems();
            a.tile_rows = out.tile_rows;
            a.t_shift = t_shift;
            // E follows D, D follows E
            if (mode == COL_RESID) {
                a.V = Ebuf; a.colmax = cmE; a.reset = cmD;
            } else {
                a.V = D; a.colmax = cmD; a.reset = cmE;
            }
            const dim3 g((unsigned)((K + COL_CHUNK - 1) / COL_CHUNK), (unsigned)B);
            switch (mode) {
                case COL_INIT: column_values_kernel<COL_INIT><<<g, 256, 0, s>>>(a); break;
                case COL_RESID: column_values_kernel<COL_RESID><<<g, 256, 0, s>>>(a); break;
                default: column_values_kernel<COL_UPDATE><<<g, 256, 0, s>>>(a); break;
            }
            count_launch();
            // phase 2 covers the padded k range of the operand's tiles
            const dim3 g2((unsigned)((out.k_tiles * split::KT + COL_CHUNK - 1) / COL_CHUNK), (unsigned)B);
            column_slices_kernel<<<g2, COL_CHUNK / 8, 0, s>>>(a);
            count_launch();
            return SMX_OK;
        };
        split::Acc acc_m{Tacc, Racc, m}, acc_n{Tacc, Racc, n};
        // U D and H^T E drop the slice pairs s + t >= 8 (U and H have no dominant
        // element per row or column: their products sit in the exact levels).
        // sh.Ut holds the slices of H^T (mixed_setup), E takes the 112-wide operand sh.Fs.
        const int sh_ud = 8 * (split::exact_levels(sh.Ua, sh.Ds) - 1);
        const int sh_he = 8 * (split::exact_levels(sh.Ut, sh.Fs) - 1);
        col(COL_INIT, n, nullptr, nullptr, sh.Ds, 0);
        for (int it = 0; it < p->maxiter; ++it) {
            if ((st = split::gemm(sh.Ua, sh.Ds, acc_m, false, derr, s, kSkinnyLevels))) return st;   // U D
            col(COL_RESID, m, sh.Ua.expo, sh.Ds.expo, sh.Fs, sh_ud);                    // E = Y - U D
            if ((st = split::gemm(sh.Ut, sh.Fs, acc_n, false, derr, s, kSkinnyLevels))) return st;   // H^T E
            col(COL_UPDATE, n, sh.Ut.expo, sh.Fs.expo, sh.Ds, sh_he);                   // ADMM update, D
        }
        SMX_TRY_CUDA(cudaMemcpyAsync(Z_out, Z, sizeof(double) * n * B, cudaMemcpyDeviceToDevice, s));
        SMX_TRY_CUDA(cudaMemcpyAsync(dinfo + 2, derr, sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    SMX_TRY_CUDA(cudaGetLastError());
    // the factorisation status is read back: a failed Cholesky is reported, not silently used
    int hinfo[4] = {0, 0, 0, 0};
    SMX_TRY_CUDA(cudaMemcpyAsync(hinfo, dinfo, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (hinfo[3] != 0) return set_error(SMX_ERR_ARGUMENT, "row_map holds an index outside [0, ld_lib)");
    if (hinfo[0] != 0) return set_error(SMX_ERR_NUMERIC, "Cholesky of rho' I + U U^T failed (info=%d)", hinfo[0]);
    if (mixed && hinfo[1] != 0)
        return set_error(SMX_ERR_NUMERIC, "inverse of rho' I + U U^T failed: a non-positive pivot of the FP32 seed or "
                         "Newton-Schulz steps that do not converge");
    if (mixed && hinfo[2] != 0) return set_error(SMX_ERR_CUDA, "split product kernel gave up waiting (code %d)", hinfo[2]);
    return SMX_OK;
}

// ------------------------------------------------------------------ jackknife
// Leave-group-out replicates of the single right-hand-side solve
// (model_deltaChi2_jackknife, model.py:480-603): replicate j raises sigma of the
// rows of its group to 1e20, i.e. drops rows d_j of U and y.  All replicates run
// as the columns of one batched ADMM and share one G^-1 of the full problem:
//   * rho_j = rho - delta_j with delta_j = ||U_dj||_F^2 / n, c_j = c - delta_j;
//   * on the kept rows K the replicate's Woodbury matrix is G_KK - delta_j I, whose
//     inverse is sum_i delta_j^i S^(i+1) (Neumann series, ||delta_j S|| <= delta_j / c)
//     with S = (G_KK)^-1 = [X - X_{:,d} (X_dd)^-1 X_{d,:}]_KK, X = G^-1 (Schur
//     complement of the dropped rows);
//   * every term is one product with the off-diagonal part O of X for all replicates
//     (split product) plus a rank-|d_j| correction per replicate.
// Dropped rows of the residual and of every term are zero, so U^T F never sees them.
// The reference's 1e-20-scaled rows differ from removed rows by 1e-40 of ||U||^2.

// row_group[r] = the replicate that drops design row r (-1: none); flag 1: a row out
// of range, 2: a row in two groups
__global__ void jk_rowgroup_kernel(const int32_t *__restrict__ drop, int max_drop, int64_t G, int64_t m,
                                   int32_t *row_group, int *flag) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < G * max_drop;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = drop[idx];
        if (r < 0) continue;
        if (r >= m) {
            atomicExch(flag, 1);
            continue;
        }
        const int32_t j = (int32_t)(idx / max_drop);
        const int32_t old = atomicCAS(row_group + r, -1, j);
        if (old != -1 && old != j) atomicExch(flag, 2);
    }
}

// ||U_r||^2 of every design row (U column-major m x n); grid (rows / 256, k splits)
__global__ void rownorm_kernel(const double *__restrict__ U, int64_t m, int64_t n, double *out) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int64_t kc = (n + gridDim.y - 1) / gridDim.y;
    const int64_t k0 = blockIdx.y * kc, k1 = k0 + kc < n ? k0 + kc : n;
    double acc = 0;
    for (int64_t i = k0; i < k1; ++i) {
        const double v = U[i * m + r];
        acc += v * v;
    }
    atomicAdd(out + r, acc);
}

constexpr int JK_MAX_DROP = 40;

// One thread per replicate: its coefficient k_j, Neumann factor delta_j, and Z_j =
// (X_dd)^-1 (Gauss-Jordan without pivoting: X_dd is symmetric positive definite).
// qmax receives max_j delta_j / c as ordered bits.
__global__ void jk_setup_kernel(const int32_t *__restrict__ drop, int max_drop, int64_t G,
                                const double *__restrict__ rownorm, const double *__restrict__ frob, double lambda,
                                double n, const double *__restrict__ O, const double *__restrict__ g, int64_t m,
                                double *kcoef, double *mu, double *Zinv, unsigned long long *qmax, int *flag) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= G) return;
    const int32_t *d = drop + j * max_drop;
    int sz = 0;
    double delta = 0;
    for (int a = 0; a < max_drop; ++a)
        if (d[a] >= 0) {
            delta += rownorm[d[a]];
            ++sz;
        }
    delta /= n;
    const double rho = (frob[0] + lambda) / n, c = rho + lambda / n;
    const double rho_j = rho - delta, c_j = c - delta;
    kcoef[j] = rho_j / c_j;
    mu[j] = delta;
    atomicMax(qmax, (unsigned long long)__double_as_longlong(delta / c));
    double *A = Zinv + j * (int64_t)max_drop * max_drop;
    // compact the dropped rows to the first sz entries of A's index space
    int idx[JK_MAX_DROP];
    int q = 0;
    for (int a = 0; a < max_drop; ++a)
        if (d[a] >= 0) idx[q++] = d[a];
    for (int a = 0; a < sz; ++a)
        for (int b = 0; b < sz; ++b)
            A[a * max_drop + b] = (a == b) ? g[idx[a]] : O[idx[a] + m * (int64_t)idx[b]];
    for (int k = 0; k < sz; ++k) {
        const double piv = A[k * max_drop + k];
        if (!(piv > 0)) {
            atomicExch(flag, 3);
            return;
        }
        const double ip = 1.0 / piv;
        for (int b = 0; b < sz; ++b) A[k * max_drop + b] *= ip;
        A[k * max_drop + k] = ip;
        for (int a = 0; a < sz; ++a) {
            if (a == k) continue;
            const double f = A[a * max_drop + k];
            if (f == 0.0) continue;
            for (int b = 0; b < sz; ++b) A[a * max_drop + b] -= f * A[k * max_drop + b];
            A[a * max_drop + k] = -f * ip;
        }
    }
}

// E = Y - U D with the replicate's dropped rows set to 0; Y is the shared data row.
// W = E starts the sum of the Neumann terms.  Grid (K / COL_CHUNK, replicates).
// T, R of the product are cleared.
__global__ void __launch_bounds__(256) jk_resid_kernel(const ColArgs a, const int32_t *__restrict__ row_group,
                                                       double *W) {
    constexpr int PER = COL_CHUNK / 256;
    const int64_t j = blockIdx.y, K = a.K;
    const int eb = a.eB[j];
    const int64_t kb = blockIdx.x * (int64_t)COL_CHUNK;
    double mx = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int64_t k = kb + threadIdx.x + q * 256, idx = k + K * j;
        if (k >= K) continue;
        const double pv = product_of((long long)a.T[idx], a.R[idx], a.eA[k], eb, a.t_shift);
        a.T[idx] = 0ull;
        a.R[idx] = 0.0f;
        const double v = row_group[k] == (int32_t)j ? 0.0 : a.Y[k] - pv;
        a.E[idx] = v;
        W[idx] = v;
        mx = fmax(mx, fabs(v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m2 = 0;
        for (int w = 0; w < 8; ++w) m2 = fmax(m2, red[w]);
        atomicMax(a.colmax + j, (unsigned long long)__double_as_longlong(m2));
    }
}

// One thread per replicate: c_j = Z_j (O V)_{d_j}  (V vanishes on d_j, so the term's
// value on the dropped rows is the product alone)
__global__ void jk_dvals_kernel(const unsigned long long *__restrict__ T, const float *__restrict__ R,
                                const int32_t *__restrict__ eA, const int32_t *__restrict__ eB, int t_shift,
                                const int32_t *__restrict__ drop, int max_drop, int64_t G, int64_t m,
                                const double *__restrict__ Zinv, double *cbuf) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= G) return;
    const int32_t *d = drop + j * max_drop;
    double pd[JK_MAX_DROP];
    int sz = 0;
    for (int a = 0; a < max_drop; ++a)
        if (d[a] >= 0) {
            const int64_t idx = d[a] + m * j;
            pd[sz++] = product_of((long long)T[idx], R[idx], eA[d[a]], eB[j], t_shift);
        }
    const double *Z = Zinv + j * (int64_t)max_drop * max_drop;
    for (int a = 0; a < sz; ++a) {
        double c = 0;
        for (int b = 0; b < sz; ++b) c += Z[a * max_drop + b] * pd[b];
        cbuf[j * max_drop + a] = c;
    }
}

// One Neumann term for every replicate, grid (K / COL_CHUNK, replicates):
//   P = g V + O V - X_{:,d} c = S V  (P = 0 on d),  V = delta_j P,  W += V,
// and the column maxima of the operand sliced next (V, or W after the last term).
__global__ void __launch_bounds__(256) jk_apply_kernel(const ColArgs a, const int32_t *__restrict__ row_group,
                                                       const int32_t *__restrict__ drop, int max_drop,
                                                       const double *__restrict__ O, const double *__restrict__ cbuf,
                                                       const double *__restrict__ mu, double *F, int last) {
    constexpr int PER = COL_CHUNK / 256;
    const int64_t j = blockIdx.y, K = a.K;
    const int eb = a.eB[j];
    __shared__ int32_t dr[JK_MAX_DROP];
    __shared__ double cc[JK_MAX_DROP];
    __shared__ int sz;
    if (threadIdx.x == 0) {
        int q = 0;
        for (int t = 0; t < max_drop; ++t) {
            const int32_t r = drop[j * max_drop + t];
            if (r >= 0) {
                dr[q] = r;
                cc[q] = cbuf[j * max_drop + q];
                ++q;
            }
        }
        sz = q;
    }
    __syncthreads();
    const double muj = mu[j];
    const int64_t kb = blockIdx.x * (int64_t)COL_CHUNK;
    double mx = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int64_t k = kb + threadIdx.x + q * 256, idx = k + K * j;
        if (k >= K) continue;
        const double pv = product_of((long long)a.T[idx], a.R[idx], a.eA[k], eb, a.t_shift);
        a.T[idx] = 0ull;
        a.R[idx] = 0.0f;
        double P = 0.0;
        if (row_group[k] != (int32_t)j) {
            P = a.g[k] * a.E[idx] + pv;
            for (int t = 0; t < sz; ++t) P -= O[k + K * (int64_t)dr[t]] * cc[t];
        }
        const double v = muj * P;
        const double f = F[idx] + v;
        F[idx] = f;
        a.E[idx] = v;
        mx = fmax(mx, fabs(last ? f : v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m2 = 0;
        for (int w = 0; w < 8; ++w) m2 = fmax(m2, red[w]);
        atomicMax(a.colmax + j, (unsigned long long)__double_as_longlong(m2));
    }
}

// Rows d_j of H = G^-1 U for every replicate, compacted: Hr[(j max_drop + q) n + i] =
// H[d + m i] for the q-th valid entry d of drop[j], 0 beyond the replicate's drops.
__global__ void jk_hrows_kernel(const double *__restrict__ H, int64_t m, int64_t n, const int32_t *__restrict__ drop,
                                int max_drop, int64_t G, double *Hr) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < G * max_drop * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t jq = idx / n, i = idx % n, j = jq / max_drop;
        const int q = (int)(jq % max_drop);
        int c = 0;
        int32_t d = -1;
        for (int t = 0; t < max_drop; ++t) {
            const int32_t r = drop[j * max_drop + t];
            if (r >= 0) {
                if (c == q) {
                    d = r;
                    break;
                }
                ++c;
            }
        }
        Hr[idx] = d >= 0 ? H[d + m * i] : 0.0;
    }
}

// c_j = (X_dd)^-1 (X W_j)_d exactly in double, one CTA per replicate: W_j vanishes
// on d, so (X W)_d = O_{d,:} W (column d of the symmetric O); cbuf[j max_drop + q]
// for the replicate's q-th drop, 0 beyond them.
__global__ void __launch_bounds__(256) jk_xdots_kernel(const double *__restrict__ O, const double *__restrict__ W,
                                                       int64_t m, const int32_t *__restrict__ drop, int max_drop,
                                                       const double *__restrict__ Zinv, double *cbuf) {
    const int64_t j = blockIdx.x;
    __shared__ double dots[JK_MAX_DROP];
    __shared__ double red[8];
    __shared__ int32_t dr[JK_MAX_DROP];
    __shared__ int sz;
    if (threadIdx.x == 0) {
        int q = 0;
        for (int t = 0; t < max_drop; ++t) {
            const int32_t r = drop[j * max_drop + t];
            if (r >= 0) dr[q++] = r;
        }
        sz = q;
    }
    __syncthreads();
    const double *w = W + m * j;
    for (int q = 0; q < sz; ++q) {
        const double *col = O + m * (int64_t)dr[q];
        double acc = 0;
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) acc += col[k] * w[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
            dots[q] = t;
        }
        __syncthreads();
    }
    if (threadIdx.x < max_drop) {
        const int q = threadIdx.x;
        double c = 0;
        if (q < sz) {
            const double *Z = Zinv + j * (int64_t)max_drop * max_drop;
            for (int b = 0; b < sz; ++b) c += Z[q * max_drop + b] * dots[b];
        }
        cbuf[j * max_drop + q] = c;
    }
}

struct JkLayout {
    size_t rownorm, kcoef, mu, Zinv, cbuf, rowgrp, qmax, flag, dummy, hrows, total;
};

static JkLayout jk_layout(size_t base, int64_t m, int64_t n, int64_t G, int max_drop) {
    JkLayout J;
    size_t off = base;
    auto take = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
    J.rownorm = take(m * sizeof(double));
    J.kcoef = take(G * sizeof(double));
    J.mu = take(G * sizeof(double));
    J.Zinv = take((size_t)G * max_drop * max_drop * sizeof(double));
    J.cbuf = take((size_t)G * max_drop * sizeof(double));
    J.rowgrp = take(m * sizeof(int32_t));
    J.qmax = take(sizeof(unsigned long long));
    J.flag = take(4 * sizeof(int));
    J.dummy = take(G * sizeof(unsigned long long));
    J.hrows = take((size_t)G * max_drop * n * sizeof(double));
    J.total = off;
    return J;
}

template <typename TL>
static int run_jackknife(const smx_nnls_problem *p, const TL *lib, const int32_t *row_map, const double *row_scale,
                         const double *Y, const int32_t *drop, int max_drop, double *Z_out, unsigned char *ws,
                         const Layout &L, const JkLayout &J, Handles *h, cudaStream_t s) {
    const int64_t m = p->m, n = p->n, B = p->n_rhs;
    double *frob = (double *)(ws + L.frob);
    int *dinfo = (int *)(ws + L.info);
    int *jflag = (int *)(ws + J.flag);
    SMX_TRY_CUDA(cudaMemsetAsync(frob, 0, sizeof(double), s));
    SMX_TRY_CUDA(cudaMemsetAsync(dinfo, 0, 4 * sizeof(int), s));
    SMX_TRY_CUDA(cudaMemsetAsync(jflag, 0, 4 * sizeof(int), s));
    MixedState S;
    int st;
    double *rownorm = (double *)(ws + J.rownorm), *kcoef = (double *)(ws + J.kcoef), *mu = (double *)(ws + J.mu);
    // the set-up with H = G^-1 U (U's row norms are taken before U is replaced by H)
    if ((st = mixed_setup<TL>(p, lib, row_map, row_scale, ws, L, h, s, S, true, rownorm))) return st;
    SplitShapes &sh = S.sh;
    double *Zinv = (double *)(ws + J.Zinv), *cbuf = (double *)(ws + J.cbuf);
    int32_t *rowgrp = (int32_t *)(ws + J.rowgrp);
    unsigned long long *qmax = (unsigned long long *)(ws + J.qmax);
    double *Hr = (double *)(ws + J.hrows);
    SMX_TRY_CUDA(cudaMemsetAsync(rowgrp, 0xff, m * sizeof(int32_t), s));
    SMX_TRY_CUDA(cudaMemsetAsync(qmax, 0, sizeof(unsigned long long), s));
    jk_rowgroup_kernel<<<grid1d(B * max_drop), 256, 0, s>>>(drop, max_drop, B, m, rowgrp, jflag);
    count_launch();
    jk_setup_kernel<<<(unsigned)((B + 63) / 64), 64, 0, s>>>(drop, max_drop, B, rownorm, frob, p->lambda_reg,
                                                             (double)n, S.Xd, S.gdiag, m, kcoef, mu, Zinv, qmax,
                                                             jflag + 1);
    count_launch();
    jk_hrows_kernel<<<grid1d(B * max_drop * n), 256, 0, s>>>(S.U, m, n, drop, max_drop, B, Hr);
    count_launch();
    // the number of Neumann terms and their slices follow the largest delta_j / c (one read-back)
    unsigned long long hq = 0;
    int hflag[4] = {0, 0, 0, 0};
    SMX_TRY_CUDA(cudaMemcpyAsync(&hq, qmax, sizeof(hq), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaMemcpyAsync(hflag, jflag, sizeof(hflag), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (hflag[0] == 1) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife: a dropped row is outside [0, m)");
    if (hflag[0] == 2) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife: a design row is dropped by two replicates");
    if (hflag[1]) return set_error(SMX_ERR_NUMERIC, "smx_nnls_jackknife: the dropped rows' block of G^-1 is not positive");
    double qv;
    memcpy(&qv, &hq, sizeof(qv));
    if (!(qv < 0.5))
        return set_error(SMX_ERR_UNSUPPORTED, "smx_nnls_jackknife: a group carries %.3g of ||U||_F^2 (at most 0.5)", qv);
    // Replicate j's update is w = D + U^T S_j W_j with W_j = sum_t (delta_j S_j)^t E_j,
    // S_j = (G_KK)^-1 (Schur complement of the dropped rows of X = G^-1).  Since W_j
    // vanishes on d_j, U^T S_j W_j = H^T W_j - H_{d,:}^T (X_dd)^-1 (X W_j)_d: one
    // product with H^T for all replicates plus a rank-|d_j| correction formed exactly.
    // Term t of W is about q^t of term 0 (q = max delta_j / c): terms follow while
    // q^t > 1e-12 (the 2^-39 slicing of the vectors), and the product of term t keeps
    // the slices that carry its 40 - t log2(1/q) significant bits.
    int terms = 1;
    for (double t = qv; t > 1e-12 && terms < 64; t *= qv) ++terms;
    const double lq = qv > 0 ? -log2(qv) : 64.0;
    double *Z = (double *)(ws + L.Z), *Uu = (double *)(ws + L.Uu), *D = (double *)(ws + L.D);
    double *Ebuf = (double *)(ws + L.Ebuf), *Wbuf = (double *)(ws + L.Fbuf);
    unsigned long long *cmD = (unsigned long long *)(ws + L.colmax), *cmE = cmD + B, *cmW = cmE + B;
    unsigned long long *dummy = (unsigned long long *)(ws + J.dummy);
    SMX_TRY_CUDA(cudaMemsetAsync(cmD, 0, 3 * B * sizeof(unsigned long long), s));
    auto args = [&](int64_t K, const int32_t *eA, const int32_t *eB, split::Operand &out, int t_shift, double *V,
                    unsigned long long *cm) {
        ColArgs a;
        memset(&a, 0, sizeof(a));
        a.K = K;
        a.n_rhs = B;
        a.T = S.Tacc;
        a.R = S.Racc;
        a.eA = eA;
        a.eB = eB;
        a.Y = Y;
        a.E = Ebuf;
        a.g = S.gdiag;
        a.Z = Z;
        a.Uu = Uu;
        a.D = D;
        a.V = V;
        a.colmax = cm;
        a.reset = dummy;
        a.coefp = frob + 1;
        a.colcoef = kcoef;
        a.w_init = p->w_init;
        a.slices = out.slices;
        a.expo = out.expo;
        a.k_tiles = out.k_tiles;
        a.slice_elems = out.slice_elems();
        a.tile_rows = out.tile_rows;
        a.t_shift = t_shift;
        return a;
    };
    auto slices = [&](const ColArgs &a, const split::Operand &out) {
        const dim3 g2((unsigned)((out.k_tiles * split::KT + COL_CHUNK - 1) / COL_CHUNK), (unsigned)B);
        column_slices_kernel<<<g2, COL_CHUNK / 8, 0, s>>>(a);
        count_launch();
    };
    split::Acc acc_m{S.Tacc, S.Racc, m}, acc_n{S.Tacc, S.Racc, n};
    const int sh_ud = 8 * (split::exact_levels(sh.Ua, sh.Ds) - 1);
    const int sh_hw = 8 * (split::exact_levels(sh.Ut, sh.Fs) - 1);
    const dim3 gm((unsigned)((m + COL_CHUNK - 1) / COL_CHUNK), (unsigned)B);
    const dim3 gn((unsigned)((n + COL_CHUNK - 1) / COL_CHUNK), (unsigned)B);
    {   // z = w_init, u = 0, D = k_j w_init, sliced
        ColArgs a = args(n, nullptr, nullptr, sh.Ds, 0, D, cmD);
        column_values_kernel<COL_INIT><<<gn, 256, 0, s>>>(a);
        count_launch();
        slices(a, sh.Ds);
    }
    for (int it = 0; it < p->maxiter; ++it) {
        if ((st = split::gemm(sh.Ua, sh.Ds, acc_m, false, S.derr, s, kSkinnyLevels))) return st;   // U D
        SMX_TRY_CUDA(cudaMemsetAsync(cmE, 0, B * sizeof(unsigned long long), s));
        {
            // E = mask(Y - U D) = W (first term); sliced as the next product's input
            split::Operand &out = terms > 1 ? sh.Es : sh.Fs;
            ColArgs a = args(m, sh.Ua.expo, sh.Ds.expo, out, sh_ud, Ebuf, cmE);
            jk_resid_kernel<<<gm, 256, 0, s>>>(a, rowgrp, Wbuf);
            count_launch();
            slices(a, out);
        }
        for (int t = 1; t < terms; ++t) {
            const bool last = t == terms - 1;
            int sl = (int)ceil((40.0 - t * lq + 1.0) / 8.0);
            sl = sl < 2 ? 2 : (sl > 5 ? 5 : sl);
            split::Operand Ot = sh.Xg, Vt = sh.Es;
            Ot.S = sl;
            Vt.S = sl;
            const int sh_ov = 8 * (split::exact_levels(Ot, Vt) - 1);
            if ((st = split::gemm(Ot, Vt, acc_m, false, S.derr, s))) return st;   // O V
            jk_dvals_kernel<<<(unsigned)((B + 127) / 128), 128, 0, s>>>(S.Tacc, S.Racc, sh.Xg.expo, sh.Es.expo, sh_ov,
                                                                        drop, max_drop, B, m, Zinv, cbuf);
            count_launch();
            unsigned long long *cm = last ? cmW : cmE;
            SMX_TRY_CUDA(cudaMemsetAsync(cm, 0, B * sizeof(unsigned long long), s));
            split::Operand &out = last ? sh.Fs : sh.Es;
            ColArgs a = args(m, sh.Xg.expo, sh.Es.expo, out, sh_ov, last ? Wbuf : Ebuf, cm);
            jk_apply_kernel<<<gm, 256, 0, s>>>(a, rowgrp, drop, max_drop, S.Xd, cbuf, mu, Wbuf, last ? 1 : 0);
            count_launch();
            slices(a, out);
        }
        if ((st = split::gemm(sh.Ut, sh.Fs, acc_n, false, S.derr, s, kSkinnyLevels))) return st;   // H^T W
        jk_xdots_kernel<<<(unsigned)B, 256, 0, s>>>(S.Xd, Wbuf, m, drop, max_drop, Zinv, cbuf);        // c_j
        count_launch();
        SMX_TRY_CUDA(cudaMemsetAsync(cmD, 0, B * sizeof(unsigned long long), s));
        {
            ColArgs a = args(n, sh.Ut.expo, sh.Fs.expo, sh.Ds, sh_hw, D, cmD);
            a.hrows = Hr;
            a.cvec = cbuf;
            a.max_drop = max_drop;
            column_values_kernel<COL_UPDATE><<<gn, 256, 0, s>>>(a);                     // ADMM update, D
            count_launch();
            slices(a, sh.Ds);
        }
    }
    SMX_TRY_CUDA(cudaMemcpyAsync(Z_out, Z, sizeof(double) * n * B, cudaMemcpyDeviceToDevice, s));
    SMX_TRY_CUDA(cudaGetLastError());
    int hinfo[4] = {0, 0, 0, 0}, herr = 0;
    SMX_TRY_CUDA(cudaMemcpyAsync(hinfo, dinfo, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaMemcpyAsync(&herr, S.derr, sizeof(int), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (hinfo[3] != 0) return set_error(SMX_ERR_ARGUMENT, "row_map holds an index outside [0, ld_lib)");
    if (hinfo[0] != 0) return set_error(SMX_ERR_NUMERIC, "Cholesky of rho' I + U U^T failed (info=%d)", hinfo[0]);
    if (hinfo[1] != 0)
        return set_error(SMX_ERR_NUMERIC, "inverse of rho' I + U U^T failed: a non-positive pivot of the FP32 seed or "
                         "Newton-Schulz steps that do not converge");
    if (herr != 0) return set_error(SMX_ERR_CUDA, "split product kernel gave up waiting (code %d)", herr);
    return SMX_OK;
}

}  // namespace smx

using namespace smx;

extern "C" int smx_nnls_workspace_size(const smx_nnls_problem *p, size_t *bytes) {
    if (!p || !bytes) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_workspace_size: NULL argument");
    if (p->n < 1 || p->m < 1 || p->n_rhs < 1) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_workspace_size: bad sizes");
    Handles *h = nullptr;
    int st = get_handles(nullptr, &h);
    if (st) return st;
    Layout L;
    st = layout(p, &L, h->solver);
    if (st) return st;
    *bytes = L.total;
    return SMX_OK;
}

extern "C" int smx_nnls_admm(const smx_nnls_problem *p, const void *library, const int32_t *row_map,
                             const double *row_scale, const double *Y, double *Z_out, void *workspace,
                             size_t workspace_bytes, void *stream) {
    if (!p) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_admm: problem is NULL");
    if (p->n < 1 || p->m < 1 || p->n_rhs < 1 || p->maxiter < 0 || p->ld_lib < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_nnls_admm: bad sizes");
    if (p->m > 46340 || p->n * p->m > ((int64_t)1 << 31) * 8)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_nnls_admm: problem too large");
    if (p->mode != SMX_NNLS_FP64 && p->mode != SMX_NNLS_MIXED)
        return set_error(SMX_ERR_ARGUMENT, "smx_nnls_admm: unknown mode %d", p->mode);
    if (!library || !row_map || !row_scale || !Y || !Z_out || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_nnls_admm: NULL buffer");
    if (!(p->lambda_reg >= 0)) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_admm: lambda must be >= 0");
    cudaStream_t s = (cudaStream_t)stream;
    Handles *h = nullptr;
    int st = get_handles(s, &h);
    if (st) return st;
    Layout L;
    st = layout(p, &L, h->solver);
    if (st) return st;
    if (workspace_bytes < L.total)
        return set_error(SMX_ERR_WORKSPACE, "smx_nnls_admm: workspace %zu < %zu bytes", workspace_bytes, L.total);
    if (p->lib_precision == SMX_FP32)
        return run<float>(p, (const float *)library, row_map, row_scale, Y, Z_out, (unsigned char *)workspace, L, h, s);
    if (p->lib_precision == SMX_FP64)
        return run<double>(p, (const double *)library, row_map, row_scale, Y, Z_out, (unsigned char *)workspace, L, h, s);
    return set_error(SMX_ERR_ARGUMENT, "bad library precision %d", p->lib_precision);
}

extern "C" int smx_nnls_jackknife_workspace_size(const smx_nnls_problem *p, int max_drop, size_t *bytes) {
    if (!p || !bytes) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife_workspace_size: NULL argument");
    if (p->n < 1 || p->m < 1 || p->n_rhs < 1 || max_drop < 1 || max_drop > JK_MAX_DROP)
        return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife_workspace_size: bad sizes");
    Handles *h = nullptr;
    int st = get_handles(nullptr, &h);
    if (st) return st;
    smx_nnls_problem q = *p;
    q.mode = SMX_NNLS_MIXED;
    Layout L;
    if ((st = layout(&q, &L, h->solver))) return st;
    *bytes = jk_layout(L.total, p->m, p->n, p->n_rhs, max_drop).total;
    return SMX_OK;
}

extern "C" int smx_nnls_jackknife(const smx_nnls_problem *p, const void *library, const int32_t *row_map,
                                  const double *row_scale, const double *Y, const int32_t *drop_rows, int max_drop,
                                  double *Z_out, void *workspace, size_t workspace_bytes, void *stream) {
    if (!p) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife: problem is NULL");
    if (p->n < 1 || p->m < 1 || p->n_rhs < 1 || p->maxiter < 0 || p->ld_lib < 1 || max_drop < 1 ||
        max_drop > JK_MAX_DROP)
        return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife: bad sizes (1 <= max_drop <= %d)", JK_MAX_DROP);
    if (p->m > 46340 || p->n * p->m > ((int64_t)1 << 31) * 8 || p->n_rhs > 65535)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_nnls_jackknife: problem too large");
    if (p->mode != SMX_NNLS_MIXED)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_nnls_jackknife: only the mixed mode (SMX_NNLS_MIXED) is batched");
    if (!library || !row_map || !row_scale || !Y || !drop_rows || !Z_out || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife: NULL buffer");
    if (!(p->lambda_reg >= 0)) return set_error(SMX_ERR_ARGUMENT, "smx_nnls_jackknife: lambda must be >= 0");
    cudaStream_t s = (cudaStream_t)stream;
    Handles *h = nullptr;
    int st = get_handles(s, &h);
    if (st) return st;
    Layout L;
    if ((st = layout(p, &L, h->solver))) return st;
    const JkLayout J = jk_layout(L.total, p->m, p->n, p->n_rhs, max_drop);
    if (workspace_bytes < J.total)
        return set_error(SMX_ERR_WORKSPACE, "smx_nnls_jackknife: workspace %zu < %zu bytes", workspace_bytes, J.total);
    unsigned char *ws = (unsigned char *)workspace;
    if (p->lib_precision == SMX_FP32)
        return run_jackknife<float>(p, (const float *)library, row_map, row_scale, Y, drop_rows, max_drop, Z_out, ws, L,
                                    J, h, s);
    if (p->lib_precision == SMX_FP64)
        return run_jackknife<double>(p, (const double *)library, row_map, row_scale, Y, drop_rows, max_drop, Z_out, ws,
                                     L, J, h, s);
    return set_error(SMX_ERR_ARGUMENT, "bad library precision %d", p->lib_precision);
}
