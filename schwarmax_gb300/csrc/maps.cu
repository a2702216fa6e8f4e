// Model maps and chi^2 per weight vector (compute_model_single, model.py:14-68;
// h_to_V_sigma, ghmoments.py:53-78; the chi^2 / log-likelihood terms of
// model_likelihood, likelihood.py:192-238).
//
// maps = W L^T is one product over all library rows.  For a float library it
// runs on the bf16 tensor cores as a split (Ozaki) product with FP64-grade
// accuracy (split_gemm.cuh): the library rows and the weight vectors in 5
// slices each (39 bits below each row's largest magnitude), so the maps carry
// no float rounding: the chi^2 summed over 100 bootstraps and several thousand
// rows moves by O(0.1) when the maps are formed in FP32 arithmetic.  A double
// library (the plain FP64 path) uses cuBLAS DGEMM.  A block per weight vector
// then forms the moments, V, sigma and the chi^2 terms and reduces them in
// double.  NaN terms are dropped as jnp.nansum does; the Rzphi term is summed
// over every weight vector and shared, as in the reference.
#include <cublas_v2.h>

#include "smx_internal.cuh"
#include "split_gemm.cuh"

namespace smx {

struct MapsLayout {
    size_t Mp, part, total;
    // split path (float library)
    split::Operand A, Bw;
    size_t a_sl, a_e, b_sl, b_e, T, R, rowmax, err;
};

static inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

static MapsLayout maps_layout(const smx_maps_problem *p) {
    MapsLayout L;
    const int64_t rows = (int64_t)p->n_cells + 6 * (int64_t)p->n_bins;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = al256(off + bytes); return o; };
    L.Mp = take((size_t)rows * p->n_rhs * sizeof(double));
    L.part = take(2 * p->n_rhs * sizeof(double));
    if (p->lib_precision == SMX_FP32) {
        L.A = split::make_operand(rows, p->n, split::MT, 5);       // library rows over orbits
        L.Bw = split::make_operand(p->n_rhs, p->n, 112, 5);        // weight vectors over orbits
        L.a_sl = take(L.A.slice_bytes());
        L.a_e = take((size_t)L.A.row_tiles * L.A.tile_rows * sizeof(int32_t));
        L.b_sl = take(L.Bw.slice_bytes());
        L.b_e = take((size_t)L.Bw.row_tiles * L.Bw.tile_rows * sizeof(int32_t));
        L.T = take((size_t)rows * p->n_rhs * sizeof(unsigned long long));
        L.R = take((size_t)rows * p->n_rhs * sizeof(float));
        L.rowmax = take((size_t)(rows > p->n_rhs ? rows : p->n_rhs) * sizeof(unsigned long long));
        L.err = take(4 * sizeof(int));
    }
    L.total = off;
    return L;
}

// Mp = 2^(eA_r + eB_b - 14) (T 2^-t_shift + R), column-major (rows x B)
__global__ void maps_combine_kernel(const unsigned long long *__restrict__ T, const float *__restrict__ R,
                                    const int32_t *__restrict__ eA, const int32_t *__restrict__ eB, double *Mp,
                                    int64_t rows, int64_t B, int t_shift) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < rows * B; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k % rows, b = k / rows;
        const double v = ldexp((double)(long long)T[k], -t_shift) + (double)R[k];
        Mp[k] = ldexp(v, eA[r] + eB[b] - 14);
    }
}

__device__ __forceinline__ double sq_or_zero_nan(double v) {
    const double q = v * v;
    return (q != q) ? 0.0 : q;   // jnp.nansum drops NaN (an inf stays)
}

template <typename TM>
__global__ void __launch_bounds__(256) maps_chi2_kernel(const TM *__restrict__ Mp, int rows, int n_cells, int nb,
                                                       const double *__restrict__ gamma, const double *__restrict__ v0,
                                                       const double *__restrict__ s, const double *__restrict__ y_rz,
                                                       const double *__restrict__ y_xy,
                                                       const double *__restrict__ y_xy_boot,
                                                       const double *__restrict__ y_h_boot,
                                                       const double *__restrict__ sig_h, int64_t B, double lum,
                                                       double amp, double *maps, double *part) {
    const int64_t b = blockIdx.x;
    const TM *col = Mp + b * rows;
    const int out_w = n_cells + 7 * nb;
    double *mo = maps ? maps + b * out_w : nullptr;
    double rz = 0, rest = 0;
    for (int c = threadIdx.x; c < n_cells; c += blockDim.x) {
        const double d3 = (double)col[c];
        if (mo) mo[c] = d3;
        rz += sq_or_zero_nan((d3 - y_rz[c]) / (0.1 * y_rz[c] * amp));
    }
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        const double surf = (double)col[n_cells + k] * lum;
        rest += sq_or_zero_nan((surf - y_xy_boot[b * nb + k]) / (0.1 * y_xy[k] * amp));
        const double g = fabs(gamma[k]) > 1e-8 ? gamma[k] : 1e-8;
        double h[4];
        for (int q = 0; q < 4; ++q) {
            double v = (double)col[n_cells + (2 + q) * nb + k] / g;
            v = v < -10.0 ? -10.0 : (v > 10.0 ? 10.0 : v);
            h[q] = v;
            rest += sq_or_zero_nan((v - y_h_boot[(q * B + b) * nb + k]) / (sig_h[q * nb + k] * amp));
        }
        if (mo) {
            const double dv = 1.4142135623730951 * h[0] + 1.7320508075688772 * h[2];
            const double s2 = 1.0 + 2.0 * 1.4142135623730951 * h[1] + 2.0 * 2.449489742783178 * h[3] - dv * dv;
            mo[n_cells + k] = surf;
            for (int q = 0; q < 4; ++q) mo[n_cells + (1 + q) * nb + k] = h[q];
            mo[n_cells + 5 * nb + k] = v0[k] + s[k] * dv;
            mo[n_cells + 6 * nb + k] = s[k] * sqrt(s2 > 1e-10 ? s2 : 1e-10);
        }
    }
    __shared__ double red[2][8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rz += __shfl_xor_sync(0xffffffffu, rz, o);
        rest += __shfl_xor_sync(0xffffffffu, rest, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = rz;
        red[1][threadIdx.x >> 5] = rest;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, c = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += red[0][w];
            c += red[1][w];
        }
        part[b] = a;
        part[B + b] = c;
    }
}

// err (optional): a nonzero code of the split product (a wait that gave up) turns
// every log-likelihood into NaN, so that a failed product is never taken for a result
__global__ void logl_kernel(const double *__restrict__ part, int64_t B, const int *err, double *logl) {
    __shared__ double tot;
    if (threadIdx.x == 0) {
        double t = 0;
        for (int64_t b = 0; b < B; ++b) t += part[b];
        tot = (err && err[0]) ? __longlong_as_double(0x7ff8000000000000ll) : t;
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < B; b += blockDim.x) logl[b] = -0.5 * (part[B + b] + tot);
}

}  // namespace smx

using namespace smx;

namespace smx {
struct BlasHandle {
    cublasHandle_t h = nullptr;
    int device = -1;
};
static thread_local BlasHandle g_maps_blas;
}  // namespace smx

extern "C" int smx_model_maps_workspace_size(const smx_maps_problem *p, size_t *bytes) {
    if (!p || !bytes) return set_error(SMX_ERR_ARGUMENT, "smx_model_maps_workspace_size: NULL argument");
    *bytes = maps_layout(p).total;
    return SMX_OK;
}

extern "C" int smx_model_maps(const smx_maps_problem *p, const void *library, const double *W,
                              const double *gamma_kin, const double *v0, const double *s, const double *y_rz,
                              const double *y_xy, const double *y_xy_boot, const double *y_h_boot,
                              const double *sig_h_raw, double *maps_out, double *logl_out, void *workspace,
                              size_t workspace_bytes, void *stream) {
    if (!p) return set_error(SMX_ERR_ARGUMENT, "smx_model_maps: problem is NULL");
    if (p->n < 1 || p->n_rhs < 1 || p->n_cells < 1 || p->n_bins < 1 ||
        p->ld_lib < (int64_t)p->n_cells + 6 * (int64_t)p->n_bins)
        return set_error(SMX_ERR_ARGUMENT, "smx_model_maps: bad sizes");
    if (!library || !W || !gamma_kin || !v0 || !s || !y_rz || !y_xy || !y_xy_boot || !y_h_boot || !sig_h_raw ||
        !logl_out || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_model_maps: NULL buffer");
    const MapsLayout L = maps_layout(p);
    if (workspace_bytes < L.total)
        return set_error(SMX_ERR_WORKSPACE, "smx_model_maps: workspace %zu < %zu bytes", workspace_bytes, L.total);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *ws = (unsigned char *)workspace;
    const int rows = p->n_cells + 6 * p->n_bins;
    const int64_t n = p->n, B = p->n_rhs;
    double *part = (double *)(ws + L.part);
    double *Mp = (double *)(ws + L.Mp);
    const int *errp = nullptr;
    if (p->lib_precision == SMX_FP32) {
        split::Operand A = L.A, Bw = L.Bw;
        A.slices = (__nv_bfloat16 *)(ws + L.a_sl);
        A.expo = (int32_t *)(ws + L.a_e);
        Bw.slices = (__nv_bfloat16 *)(ws + L.b_sl);
        Bw.expo = (int32_t *)(ws + L.b_e);
        unsigned long long *T = (unsigned long long *)(ws + L.T);
        float *R = (float *)(ws + L.R);
        int *err = (int *)(ws + L.err);
        SMX_TRY_CUDA(cudaMemsetAsync(T, 0, (size_t)rows * B * sizeof(unsigned long long), st));
        SMX_TRY_CUDA(cudaMemsetAsync(R, 0, (size_t)rows * B * sizeof(float), st));
        SMX_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        unsigned long long *rowmax = (unsigned long long *)(ws + L.rowmax);
        int sst;
        // library element (row r, orbit i) at lib[i ld + r];  W element (b, i) at W[b n + i]
        if ((sst = split::slice_rows<float>((const float *)library, 1, p->ld_lib, A, rowmax, st))) return sst;
        if ((sst = split::slice_rows<double>(W, n, 1, Bw, rowmax, st))) return sst;
        split::Acc acc{T, R, rows};
        if ((sst = split::gemm(A, Bw, acc, false, err, st))) return sst;
        const int64_t cnt = (int64_t)rows * B;
        maps_combine_kernel<<<(unsigned)((cnt + 255) / 256 < 4864 ? (cnt + 255) / 256 : 4864), 256, 0, st>>>(
            T, R, A.expo, Bw.expo, Mp, rows, B, 8 * (split::exact_levels(A, Bw) - 1));
        count_launch();
        maps_chi2_kernel<double><<<(unsigned)B, 256, 0, st>>>(Mp, rows, p->n_cells, p->n_bins, gamma_kin, v0, s, y_rz,
                                                             y_xy, y_xy_boot, y_h_boot, sig_h_raw, B, p->lum_factor,
                                                             p->sigma_amplify, maps_out, part);
        count_launch();
        errp = err;
    } else if (p->lib_precision == SMX_FP64) {
        int dev = 0;
        SMX_TRY_CUDA(cudaGetDevice(&dev));
        if (g_maps_blas.device != dev) {
            if (g_maps_blas.h) cublasDestroy(g_maps_blas.h);
            if (cublasCreate(&g_maps_blas.h) != CUBLAS_STATUS_SUCCESS)
                return set_error(SMX_ERR_CUDA, "cublasCreate failed");
            g_maps_blas.device = dev;
        }
        cublasHandle_t h = g_maps_blas.h;
        cublasSetStream(h, st);
        cublasSetMathMode(h, CUBLAS_DEFAULT_MATH);
        const double one = 1.0, zero = 0.0;
        cublasStatus_t bs = cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, rows, (int)B, (int)n, &one,
                                        (const double *)library, (int)p->ld_lib, W, (int)n, &zero, Mp, rows);
        if (bs != CUBLAS_STATUS_SUCCESS) return set_error(SMX_ERR_CUDA, "cublasDgemm (maps) status %d", (int)bs);
        maps_chi2_kernel<double><<<(unsigned)B, 256, 0, st>>>(Mp, rows, p->n_cells, p->n_bins, gamma_kin, v0, s, y_rz,
                                                             y_xy, y_xy_boot, y_h_boot, sig_h_raw, B, p->lum_factor,
                                                             p->sigma_amplify, maps_out, part);
        count_launch();
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad library precision %d", p->lib_precision);
    }
    logl_kernel<<<1, 128, 0, st>>>(part, B, errp, logl_out);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}
