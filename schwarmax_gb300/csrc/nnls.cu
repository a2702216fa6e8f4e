// ADMM non-negative least squares for many right-hand sides
// (solve_nnls_admm_bootstrap, nnls.py:68-166; solve_nnls_admm, nnls.py:6-66).
//
// The reference factorises the n x n matrix Q + rho I = U^T U + (lambda/n + rho) I.
// The design matrix has fewer rows than columns (m < n), so the same inverse
// is applied through the Woodbury identity with the m x m matrix
//   G = c I + U U^T,   c = rho + lambda/n,   rho = (||U||_F^2 + lambda)/n:
//   (Q + rho I)^-1 v = (v - U^T G^-1 U v) / c.
// With d = z - u the ADMM update w = (Q + rho I)^-1 (rho d + U^T y) becomes
//   w = (rho/c) (d - U^T G^-1 U d) + U^T G^-1 y,
// so each iteration costs two skinny GEMMs with U and one application of G^-1;
// U^T G^-1 y is formed once.  Then w^ = 1.6 w - 0.6 z, z = max(0, w^ + u),
// u = u + w^ - z exactly as nnls.py:151-158.
//
// SMX_NNLS_FP64: every step in double (cuBLAS DSYRK/DGEMM, cuSOLVER DPOTRF/DPOTRS).
// SMX_NNLS_MIXED: U in float; G = U U^T on the tensor cores (TF32 inputs, FP32
// accumulation); ||U||_F^2, G + cI and its Cholesky factor in double; G^-1 is
// formed once in float from the double factor and the iterations run float
// GEMMs on the tensor cores.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cstdio>

#include "smx_internal.cuh"

namespace smx {

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

struct Layout {
    size_t U, G, Gf, work, info, frob, V, Vf, Wc, Z, Uu, D, E, F, Gt, total;
    int lwork;
};

static int layout(const smx_nnls_problem *p, Layout *L, cusolverDnHandle_t solver) {
    const size_t m = p->m, n = p->n, B = p->n_rhs;
    const bool mixed = p->mode == SMX_NNLS_MIXED;
    const size_t eu = mixed ? sizeof(float) : sizeof(double);   // U and iteration element size
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
    L->U = take(m * n * eu);
    L->G = take(m * m * sizeof(double));
    L->Gf = mixed ? take(m * m * sizeof(float)) : 0;
    int lwork = 0;
    if (solver) {
        SMX_TRY_SOLVER(cusolverDnDpotrf_bufferSize(solver, CUBLAS_FILL_MODE_LOWER, (int)m, nullptr, (int)m, &lwork));
    } else {
        lwork = (int)(m * 256 + (1 << 20));   // generous estimate for size queries without a handle
    }
    L->lwork = lwork;
    L->work = take((size_t)lwork * sizeof(double));
    L->info = take(sizeof(int) * 4);
    L->frob = take(sizeof(double) * 4);   // ||U||_F^2, coef (double), coef (float)
    L->V = take(m * B * sizeof(double));
    L->Vf = mixed ? take(m * B * sizeof(float)) : 0;
    L->Wc = take(n * B * eu);
    L->Z = take(n * B * eu);
    L->Uu = take(n * B * eu);
    L->D = take(n * B * eu);
    L->E = take(m * B * eu);
    L->F = take(m * B * eu);
    L->Gt = take(n * B * eu);
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

// G (double, lower part used) = Gsrc + c I, where c = (frob + lambda)/n + lambda/n
template <typename TS>
__global__ void shift_gram_kernel(const TS *__restrict__ Gsrc, double *G, int64_t m, const double *frob,
                                  double lambda, double n) {
    const double rho = (frob[0] + lambda) / n;
    const double c = rho + lambda / n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * m; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k % m, j = k / m;
        double v = (double)Gsrc[k];
        if (i == j) v += c;
        G[k] = v;
    }
}

__global__ void add_diag_kernel(double *G, int64_t m, const double *frob, double lambda, double n) {
    const double c = (frob[0] + lambda) / n + lambda / n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        G[i * m + i] += c;
}

template <typename TO>
__global__ void convert_kernel(const double *__restrict__ src, TO *dst, int64_t count) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x)
        dst[k] = TO(src[k]);
}

// lower-triangular copy of the double factor into float with zeros above
__global__ void tril_to_float_kernel(const double *__restrict__ L, float *Lf, int64_t m) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * m; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k % m, j = k / m;
        Lf[k] = i >= j ? float(L[k]) : 0.0f;
    }
}

__global__ void identity_kernel(float *X, int64_t m) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m * m; k += (int64_t)gridDim.x * blockDim.x)
        X[k] = (k % m == k / m) ? 1.0f : 0.0f;
}

template <typename T>
__global__ void admm_init_kernel(T *Z, T *Uu, T *D, int64_t count, double w_init) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        Z[k] = T(w_init);
        Uu[k] = T(0);
        D[k] = T(w_init);
    }
}

// coef[0] = rho / (rho + lambda/n) with rho = (||U||_F^2 + lambda)/n, in double and float
__global__ void admm_coef_kernel(const double *frob, double lambda, double n, double *coef) {
    const double rho = (frob[0] + lambda) / n;
    coef[0] = rho / (rho + lambda / n);
    ((float *)(coef + 1))[0] = (float)coef[0];
}

// w = (rho/c)(d - g) + wc;  w^ = 1.6 w - 0.6 z;  z = max(0, w^ + u);  u += w^ - z;  d = z - u
template <typename T>
__global__ void admm_update_kernel(const T *__restrict__ Gt, const T *__restrict__ Wc, T *Z, T *Uu, T *D,
                                   int64_t count, const double *coefp) {
    const T coef = sizeof(T) == 8 ? T(coefp[0]) : T(((const float *)(coefp + 1))[0]);
    const T alpha = T(1.6);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        const T z = Z[k], u = Uu[k];
        const T w = coef * (D[k] - Gt[k]) + Wc[k];
        const T wh = alpha * w + (T(1) - alpha) * z;
        T zn = wh + u;
        zn = zn > T(0) ? zn : T(0);
        const T un = u + wh - zn;
        Z[k] = zn;
        Uu[k] = un;
        D[k] = zn - un;
    }
}

__global__ void f2d_kernel(const float *src, double *dst, int64_t count) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x)
        dst[k] = (double)src[k];
}

static inline unsigned grid1d(int64_t count, int bs = 256) {
    int64_t g = (count + bs - 1) / bs;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return (unsigned)g;
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
    double *V = (double *)(ws + L.V);
    SMX_TRY_CUDA(cudaMemsetAsync(frob, 0, sizeof(double), s));
    SMX_TRY_CUDA(cudaMemsetAsync(dinfo, 0, 4 * sizeof(int), s));
    dim3 gb((unsigned)((m + 255) / 256 < 65535 ? (m + 255) / 256 : 65535), (unsigned)(n < 65535 ? n : 65535));
    const double one = 1.0, zero = 0.0;
    const float onef = 1.0f, zerof = 0.0f;
    if (!mixed) {
        double *U = (double *)(ws + L.U);
        build_u_kernel<TL, double><<<gb, 256, 0, s>>>(lib, p->ld_lib, row_map, row_scale, m, n, U, dinfo + 3);
        count_launch();
        frob_kernel<double><<<grid1d(m * n), 256, 0, s>>>(U, m * n, frob);
        count_launch();
        admm_coef_kernel<<<1, 1, 0, s>>>(frob, lam, (double)n, frob + 1);
        count_launch();
        SMX_TRY_BLAS(cublasSetMathMode(h->blas, CUBLAS_DEFAULT_MATH));
        SMX_TRY_BLAS(cublasDsyrk(h->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, (int)m, (int)n, &one, U, (int)m, &zero,
                                 G, (int)m));
        add_diag_kernel<<<grid1d(m), 256, 0, s>>>(G, m, frob, lam, (double)n);
        count_launch();
        SMX_TRY_SOLVER(cusolverDnDpotrf(h->solver, CUBLAS_FILL_MODE_LOWER, (int)m, G, (int)m, (double *)(ws + L.work),
                                        L.lwork, dinfo));
        SMX_TRY_CUDA(cudaMemcpyAsync(V, Y, sizeof(double) * m * B, cudaMemcpyDeviceToDevice, s));
        SMX_TRY_SOLVER(cusolverDnDpotrs(h->solver, CUBLAS_FILL_MODE_LOWER, (int)m, (int)B, G, (int)m, V, (int)m, dinfo + 1));
        double *Wc = (double *)(ws + L.Wc), *Z = (double *)(ws + L.Z), *Uu = (double *)(ws + L.Uu),
               *D = (double *)(ws + L.D), *E = (double *)(ws + L.E), *Gt = (double *)(ws + L.Gt);
        SMX_TRY_BLAS(cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)B, (int)m, &one, U, (int)m, V, (int)m,
                                 &zero, Wc, (int)n));
        admm_init_kernel<double><<<grid1d(n * B), 256, 0, s>>>(Z, Uu, D, n * B, p->w_init);
        count_launch();
        for (int it = 0; it < p->maxiter; ++it) {
            SMX_TRY_BLAS(cublasDgemm(h->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, (int)B, (int)n, &one, U, (int)m, D,
                                     (int)n, &zero, E, (int)m));
            SMX_TRY_SOLVER(cusolverDnDpotrs(h->solver, CUBLAS_FILL_MODE_LOWER, (int)m, (int)B, G, (int)m, E, (int)m,
                                            dinfo + 2));
            SMX_TRY_BLAS(cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)B, (int)m, &one, U, (int)m, E,
                                     (int)m, &zero, Gt, (int)n));
            admm_update_kernel<double><<<grid1d(n * B), 256, 0, s>>>(Gt, Wc, Z, Uu, D, n * B, frob + 1);
            count_launch();
        }
        SMX_TRY_CUDA(cudaMemcpyAsync(Z_out, Z, sizeof(double) * n * B, cudaMemcpyDeviceToDevice, s));
    } else {
        float *U = (float *)(ws + L.U);
        float *Gf = (float *)(ws + L.Gf);
        build_u_kernel<TL, float><<<gb, 256, 0, s>>>(lib, p->ld_lib, row_map, row_scale, m, n, U, dinfo + 3);
        count_launch();
        frob_kernel<float><<<grid1d(m * n), 256, 0, s>>>(U, m * n, frob);
        count_launch();
        admm_coef_kernel<<<1, 1, 0, s>>>(frob, lam, (double)n, frob + 1);
        count_launch();
        SMX_TRY_BLAS(cublasSetMathMode(h->blas, CUBLAS_TF32_TENSOR_OP_MATH));
        SMX_TRY_BLAS(cublasGemmEx(h->blas, CUBLAS_OP_N, CUBLAS_OP_T, (int)m, (int)m, (int)n, &onef, U, CUDA_R_32F,
                                  (int)m, U, CUDA_R_32F, (int)m, &zerof, Gf, CUDA_R_32F, (int)m,
                                  CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT));
        shift_gram_kernel<float><<<grid1d(m * m), 256, 0, s>>>(Gf, G, m, frob, lam, (double)n);
        count_launch();
        SMX_TRY_SOLVER(cusolverDnDpotrf(h->solver, CUBLAS_FILL_MODE_LOWER, (int)m, G, (int)m, (double *)(ws + L.work),
                                        L.lwork, dinfo));
        float *Wc = (float *)(ws + L.Wc), *Z = (float *)(ws + L.Z), *Uu = (float *)(ws + L.Uu),
              *D = (float *)(ws + L.D), *E = (float *)(ws + L.E), *F = (float *)(ws + L.F), *Gt = (float *)(ws + L.Gt);
        // G^-1 in float from the double factor: Lf = tril(L), Linv = L^-1 by TRSM on the
        // identity, G^-1 = Linv^T Linv.  G's double storage holds the two float m x m
        // matrices once the factor has been copied out.
        float *Lf = Gf;
        tril_to_float_kernel<<<grid1d(m * m), 256, 0, s>>>(G, Lf, m);
        count_launch();
        float *Linv = (float *)G;
        float *Gi = (float *)G + m * m;
        identity_kernel<<<grid1d(m * m), 256, 0, s>>>(Linv, m);
        count_launch();
        SMX_TRY_BLAS(cublasSetMathMode(h->blas, CUBLAS_DEFAULT_MATH));
        SMX_TRY_BLAS(cublasStrsm(h->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                                 (int)m, (int)m, &onef, Lf, (int)m, Linv, (int)m));
        SMX_TRY_BLAS(cublasSgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)m, (int)m, (int)m, &onef, Linv, (int)m, Linv,
                                 (int)m, &zerof, Gi, (int)m));
        // constant term Wc = U^T G^-1 Y with the same G^-1 the iterations use (FP32)
        convert_kernel<float><<<grid1d(m * B), 256, 0, s>>>(Y, E, m * B);
        count_launch();
        SMX_TRY_BLAS(cublasSgemm(h->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, (int)B, (int)m, &onef, Gi, (int)m, E, (int)m,
                                 &zerof, F, (int)m));
        SMX_TRY_BLAS(cublasSgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)B, (int)m, &onef, U, (int)m, F,
                                 (int)m, &zerof, Wc, (int)n));
        admm_init_kernel<float><<<grid1d(n * B), 256, 0, s>>>(Z, Uu, D, n * B, p->w_init);
        count_launch();
        SMX_TRY_BLAS(cublasSetMathMode(h->blas, CUBLAS_TF32_TENSOR_OP_MATH));
        for (int it = 0; it < p->maxiter; ++it) {
            SMX_TRY_BLAS(cublasGemmEx(h->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, (int)B, (int)n, &onef, U, CUDA_R_32F,
                                      (int)m, D, CUDA_R_32F, (int)n, &zerof, E, CUDA_R_32F, (int)m,
                                      CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT));
            SMX_TRY_BLAS(cublasGemmEx(h->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, (int)B, (int)m, &onef, Gi, CUDA_R_32F,
                                      (int)m, E, CUDA_R_32F, (int)m, &zerof, F, CUDA_R_32F, (int)m,
                                      CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT));
            SMX_TRY_BLAS(cublasGemmEx(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)B, (int)m, &onef, U, CUDA_R_32F,
                                      (int)m, F, CUDA_R_32F, (int)m, &zerof, Gt, CUDA_R_32F, (int)n,
                                      CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT));
            admm_update_kernel<float><<<grid1d(n * B), 256, 0, s>>>(Gt, Wc, Z, Uu, D, n * B, frob + 1);
            count_launch();
        }
        SMX_TRY_BLAS(cublasSetMathMode(h->blas, CUBLAS_DEFAULT_MATH));
        f2d_kernel<<<grid1d(n * B), 256, 0, s>>>(Z, Z_out, n * B);
        count_launch();
    }
    SMX_TRY_CUDA(cudaGetLastError());
    // the factorisation status is read back: a failed Cholesky is reported, not silently used
    int hinfo[4] = {0, 0, 0, 0};
    SMX_TRY_CUDA(cudaMemcpyAsync(hinfo, dinfo, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (hinfo[3] != 0) return set_error(SMX_ERR_ARGUMENT, "row_map holds an index outside [0, ld_lib)");
    if (hinfo[0] != 0) return set_error(SMX_ERR_NUMERIC, "Cholesky of rho' I + U U^T failed (info=%d)", hinfo[0]);
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
