// Post-analysis of an evaluation on the device:
//   * the circular-orbit table of build_Lcirc_of_E (utils.py:275-341) and the
//     circularity lambda_z = L_z / L_circ(E) of every stored sample
//     (example/example_analysis.ipynb, model-side circularity cell), with a
//     weighted 2-D histogram laid out like np.histogram2d;
//   * the PSF transfer matrix of compute_transfer_matrix (utils.py:413-485).
#include "smx_internal.cuh"

namespace smx {

// midplane circular-orbit table: R_i log-spaced, Phi(R_i, 0, 0) and the central
// difference of Phi along x (utils.py:322-333), all in double
__global__ void lcirc_table_kernel(PotT<double> P, double lR0, double lR1, double dlR, int n, double dR, double *E,
                                   double *L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // np.logspace: 10 ** (i step + start), the last exponent exactly log10 R_max
    // (explicitly rounded operations: no contraction into an FMA)
    const double ex = (i == n - 1) ? lR1 : __dadd_rn(__dmul_rn((double)i, dlR), lR0);
    const double R = pow(10.0, ex);
    const double ph = phi_only(P, R, 0.0, 0.0);
    const double pp = phi_only(P, __dadd_rn(R, dR), 0.0, 0.0);
    const double pm = phi_only(P, __dsub_rn(R, dR), 0.0, 0.0);
    const double d = __ddiv_rn(__dsub_rn(pp, pm), __dmul_rn(2.0, dR));
    const double vc2 = fmax(__dmul_rn(R, d), 0.0);
    E[i] = __dadd_rn(ph, __dmul_rn(0.5, vc2));
    L[i] = __dmul_rn(R, sqrt(vc2));
}

// cubic spline value at e: knots k (n), coefficients c (4, n-1) in powers of (e - k_j),
// highest first; clamped to the end values outside [k_0, k_{n-1}] (interp1d with
// fill_value = (L[0], L[-1]))
__device__ __forceinline__ double spline_eval(const double *__restrict__ k, const double *__restrict__ c, int n,
                                              double e, double below, double above) {
    if (e != e) return e;
    if (e < k[0]) return below;
    if (e > k[n - 1]) return above;
    int lo = 0, hi = n - 1;   // k[lo] <= e <= k[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (k[mid] <= e) lo = mid;
        else hi = mid;
    }
    const double t = e - k[lo];
    return ((c[lo] * t + c[(n - 1) + lo]) * t + c[2 * (n - 1) + lo]) * t + c[3 * (n - 1) + lo];
}

__global__ void spline_eval_kernel(const double *__restrict__ k, const double *__restrict__ c, int n, double below,
                                   double above, const double *__restrict__ x, int64_t N, double *out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) out[i] = spline_eval(k, c, n, x[i], below, above);
}

template <typename T>
__global__ void circularity_kernel(PotT<T> P, const T *__restrict__ pts, int64_t N, const double *__restrict__ knots,
                                   const double *__restrict__ coef, int n_knots, double below, double above, T *lam,
                                   T *Rout, T *Eout) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    const T x = pts[i], y = pts[N + i], z = pts[2 * N + i];
    const T vx = pts[3 * N + i], vy = pts[4 * N + i], vz = pts[5 * N + i];
    const T E = T(0.5) * (vx * vx + vy * vy + vz * vz) + phi_only(P, x, y, z);
    const T Lz = -(x * vy - y * vx);
    const double Lc = spline_eval(knots, coef, n_knots, (double)E, below, above);
    if (lam) lam[i] = Lz / (T(Lc) + T(1e-10));
    if (Rout) Rout[i] = sqrt(x * x + y * y);
    if (Eout) Eout[i] = E;
}

// np.histogram2d bin of v over edges e (n + 1, increasing): searchsorted(side='right')
// - 1, with v == e[n] in the last bin; -1 outside
__device__ __forceinline__ int hist_bin(const double *__restrict__ e, int n, double v) {
    if (!(v >= e[0]) || !(v <= e[n])) return -1;
    if (v == e[n]) return n - 1;
    int lo = 0, hi = n;   // e[lo] <= v < e[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

// weighted histogram as exact int64 fixed point (units 2^-40 of the weight scale)
template <typename T>
__global__ void histogram2d_kernel(const T *__restrict__ a, const T *__restrict__ b, const T *__restrict__ w, int64_t N,
                                   const double *__restrict__ ea, int na, const double *__restrict__ eb, int nb,
                                   double inv_scale, unsigned long long *acc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int ia = hist_bin(ea, na, (double)a[i]);
        const int ib = hist_bin(eb, nb, (double)b[i]);
        if (ia < 0 || ib < 0) continue;
        const double wv = w ? (double)w[i] : 1.0;
        red_add(acc + (int64_t)ia * nb + ib, (unsigned long long)__double2ll_rn(wv * inv_scale * 0x1p40));
    }
}

__global__ void fixed_to_double_kernel(const unsigned long long *__restrict__ acc, int64_t n, double scale,
                                       double *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)(long long)acc[i] * 0x1p-40 * scale;
}

// ---------------------------------------------------------------- PSF transfer
// Fine grid point (gx, gy) -> Voronoi bin through the nX x nY pixel map, in the
// arithmetic of utils.py:451-463 (np.linspace edges, centres, floor, clip).
__global__ void fine_bins_kernel(int grid_res, double X_lo, double X_hi, double Y_lo, double Y_hi, int nX, int nY,
                                 const int32_t *__restrict__ bin_mapping, int32_t *fine) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= (int64_t)grid_res * grid_res) return;
    const int gx = (int)(p % grid_res), gy = (int)(p / grid_res);
    const double sx = (X_hi - X_lo) / grid_res, sy = (Y_hi - Y_lo) / grid_res;
    // np.linspace edges i step + start (last edge exact), rounded once per operation
    const double x0 = __dadd_rn(__dmul_rn((double)gx, sx), X_lo);
    const double x1 = (gx + 1 == grid_res) ? X_hi : __dadd_rn(__dmul_rn((double)(gx + 1), sx), X_lo);
    const double y0 = __dadd_rn(__dmul_rn((double)gy, sy), Y_lo);
    const double y1 = (gy + 1 == grid_res) ? Y_hi : __dadd_rn(__dmul_rn((double)(gy + 1), sy), Y_lo);
    const double xc = 0.5 * (x0 + x1), yc = 0.5 * (y0 + y1);
    const double nx = (xc - X_lo) / (X_hi - X_lo), ny = (yc - Y_lo) / (Y_hi - Y_lo);
    int ix = (int)floor(nx * nX), iy = (int)floor(ny * nY);
    ix = ix < 0 ? 0 : (ix > nX - 1 ? nX - 1 : ix);
    iy = iy < 0 ? 0 : (iy > nY - 1 ? nY - 1 : iy);
    fine[p] = bin_mapping[ix + iy * nX];
}

constexpr int PSF_MAX_BINS = 16;   // distinct bins in one row window of a fine point

// Stage 1 (rows): for every fine point p, the bins met along its row within the
// kernel radius, each with its summed weight k(dx).  Stage 2 (columns): every fine
// point q in bin i adds k(dy) * (row sums of the point dy below/above) to P[i, j].
// Both sums are exact int64 fixed point, so P does not depend on the order of adds.
__global__ void psf_rows_kernel(int grid_res, int radius, const double *__restrict__ kw,
                                const int32_t *__restrict__ fine, int32_t *rb, double *rw, int *flag) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= (int64_t)grid_res * grid_res) return;
    const int gx = (int)(p % grid_res);
    const int64_t row0 = p - gx;
    int nb = 0;
    int32_t bins[PSF_MAX_BINS];
    double ws[PSF_MAX_BINS];
    for (int dx = -radius; dx <= radius; ++dx) {
        const int qx = gx + dx;
        if (qx < 0 || qx >= grid_res) continue;
        const int32_t b = fine[row0 + qx];
        if (b < 0) continue;
        int t = 0;
        while (t < nb && bins[t] != b) ++t;
        if (t == nb) {
            if (nb == PSF_MAX_BINS) {
                atomicExch(flag, 1);
                continue;
            }
            bins[nb] = b;
            ws[nb] = 0.0;
            ++nb;
        }
        ws[t] += kw[dx + radius];
    }
    for (int t = 0; t < PSF_MAX_BINS; ++t) {
        rb[p * PSF_MAX_BINS + t] = t < nb ? bins[t] : -1;
        rw[p * PSF_MAX_BINS + t] = t < nb ? ws[t] : 0.0;
    }
}

__global__ void psf_cols_kernel(int grid_res, int radius, const double *__restrict__ kw,
                                const int32_t *__restrict__ fine, const int32_t *__restrict__ rb,
                                const double *__restrict__ rw, int total_bins, unsigned long long *acc) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= (int64_t)grid_res * grid_res) return;
    const int32_t i = fine[q];
    if (i < 0) return;
    const int gx = (int)(q % grid_res), gy = (int)(q / grid_res);
    for (int dy = -radius; dy <= radius; ++dy) {
        const int py = gy + dy;
        if (py < 0 || py >= grid_res) continue;
        const int64_t p = (int64_t)py * grid_res + gx;
        const double k = kw[dy + radius];
        for (int t = 0; t < PSF_MAX_BINS; ++t) {
            const int32_t j = rb[p * PSF_MAX_BINS + t];
            if (j < 0) break;
            // P[i, j] row-major, as the reference's (total_bins, total_bins) array
            red_add(acc + (int64_t)i * total_bins + j, (unsigned long long)__double2ll_rn(k * rw[p * PSF_MAX_BINS + t] *
                                                                                         0x1p40));
        }
    }
}

// column sums and normalisation: P[:, j] /= sum_i P[i, j] (columns with zero sum stay)
__global__ void psf_normalise_kernel(const unsigned long long *__restrict__ acc, int total_bins, double *P) {
    const int j = blockIdx.x;
    __shared__ long long part[256];
    long long s = 0;
    for (int i = threadIdx.x; i < total_bins; i += blockDim.x) s += (long long)acc[(int64_t)i * total_bins + j];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    const double tot = (double)part[0] * 0x1p-40;
    const double d = tot > 0 ? tot : 1.0;
    for (int i = threadIdx.x; i < total_bins; i += blockDim.x)
        P[(int64_t)i * total_bins + j] = (double)(long long)acc[(int64_t)i * total_bins + j] * 0x1p-40 / d;
}

static inline unsigned blocks_for(int64_t n, int bs) {
    int64_t g = (n + bs - 1) / bs;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace smx

using namespace smx;

extern "C" int smx_lcirc_table(const smx_potential *pot, double R_min, double R_max, int n_grid, double dR, double *E_out,
                               double *L_out, void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (!(R_min > 0) || !(R_max > R_min) || n_grid < 2 || !(dR > 0) || !E_out || !L_out)
        return set_error(SMX_ERR_ARGUMENT, "smx_lcirc_table: bad arguments");
    const double l0 = log10(R_min), l1 = log10(R_max);
    lcirc_table_kernel<<<blocks_for(n_grid, 128), 128, 0, (cudaStream_t)stream>>>(
        make_pot<double>(*pot), l0, l1, (l1 - l0) / (n_grid - 1), n_grid, dR, E_out, L_out);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

extern "C" int smx_circularity(const smx_potential *pot, int precision, const void *points, int64_t n,
                               const double *knots, const double *coef, int n_knots, double L_below, double L_above,
                               void *lam, void *R, void *E, void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (n < 0 || n_knots < 2) return set_error(SMX_ERR_ARGUMENT, "smx_circularity: bad sizes");
    if (n == 0) return SMX_OK;
    if (!points || !knots || !coef) return set_error(SMX_ERR_ARGUMENT, "smx_circularity: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == SMX_FP32) {
        circularity_kernel<float><<<blocks_for(n, 256), 256, 0, s>>>(make_pot<float>(*pot), (const float *)points, n,
                                                                     knots, coef, n_knots, L_below, L_above,
                                                                     (float *)lam, (float *)R, (float *)E);
    } else if (precision == SMX_FP64) {
        circularity_kernel<double><<<blocks_for(n, 256), 256, 0, s>>>(make_pot<double>(*pot), (const double *)points,
                                                                      n, knots, coef, n_knots, L_below, L_above,
                                                                      (double *)lam, (double *)R, (double *)E);
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

extern "C" int smx_spline_eval(const double *knots, const double *coef, int n_knots, double below, double above,
                               const double *x, int64_t n, double *out, void *stream) {
    if (n < 0 || n_knots < 2) return set_error(SMX_ERR_ARGUMENT, "smx_spline_eval: bad sizes");
    if (n == 0) return SMX_OK;
    if (!knots || !coef || !x || !out) return set_error(SMX_ERR_ARGUMENT, "smx_spline_eval: NULL buffer");
    spline_eval_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(knots, coef, n_knots, below, above, x, n,
                                                                            out);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

extern "C" int smx_histogram2d(int precision, const void *a, const void *b, const void *w, int64_t n,
                               const double *edges_a, int na, const double *edges_b, int nb, double weight_scale,
                               unsigned long long *scratch, double *out, void *stream) {
    if (n < 0 || na < 1 || nb < 1 || !(weight_scale > 0)) return set_error(SMX_ERR_ARGUMENT, "smx_histogram2d: bad sizes");
    if (!a || !b || !edges_a || !edges_b || !scratch || !out) return set_error(SMX_ERR_ARGUMENT, "smx_histogram2d: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t cells = (int64_t)na * nb;
    SMX_TRY_CUDA(cudaMemsetAsync(scratch, 0, cells * sizeof(unsigned long long), s));
    if (n > 0) {
        const unsigned g = (unsigned)(n / 256 + 1 < 152 * 16 ? n / 256 + 1 : 152 * 16);
        if (precision == SMX_FP32)
            histogram2d_kernel<float><<<g, 256, 0, s>>>((const float *)a, (const float *)b, (const float *)w, n, edges_a,
                                                        na, edges_b, nb, 1.0 / weight_scale, scratch);
        else if (precision == SMX_FP64)
            histogram2d_kernel<double><<<g, 256, 0, s>>>((const double *)a, (const double *)b, (const double *)w, n,
                                                         edges_a, na, edges_b, nb, 1.0 / weight_scale, scratch);
        else
            return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
        count_launch();
    }
    fixed_to_double_kernel<<<blocks_for(cells, 256), 256, 0, s>>>(scratch, cells, weight_scale, out);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

extern "C" int smx_psf_transfer_workspace_size(int grid_res, int total_bins, int radius, size_t *bytes) {
    if (!bytes || grid_res < 1 || total_bins < 1 || radius < 0)
        return set_error(SMX_ERR_ARGUMENT, "smx_psf_transfer_workspace_size: bad arguments");
    const size_t pts = (size_t)grid_res * grid_res;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    *bytes = al(pts * sizeof(int32_t)) + al(pts * PSF_MAX_BINS * sizeof(int32_t)) +
             al(pts * PSF_MAX_BINS * sizeof(double)) + al((size_t)total_bins * total_bins * 8) +
             al((2 * (size_t)radius + 1) * sizeof(double)) + al(4 * sizeof(int));
    return SMX_OK;
}

extern "C" int smx_psf_transfer(const double *kernel_weights, int radius, int nX, int nY, double X_lo, double X_hi,
                                double Y_lo, double Y_hi, const int32_t *bin_mapping, int total_bins, int grid_res,
                                double *P, void *workspace, size_t workspace_bytes, void *stream) {
    if (!kernel_weights || radius < 0 || nX < 1 || nY < 1 || !(X_hi > X_lo) || !(Y_hi > Y_lo) || !bin_mapping ||
        total_bins < 1 || grid_res < 1 || !P || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_psf_transfer: bad arguments");
    if ((int64_t)grid_res * grid_res * PSF_MAX_BINS > ((int64_t)1 << 31))
        return set_error(SMX_ERR_UNSUPPORTED, "smx_psf_transfer: grid_res too large");
    size_t need = 0;
    int st = smx_psf_transfer_workspace_size(grid_res, total_bins, radius, &need);
    if (st) return st;
    if (workspace_bytes < need)
        return set_error(SMX_ERR_WORKSPACE, "smx_psf_transfer: workspace %zu < %zu bytes", workspace_bytes, need);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t pts = (size_t)grid_res * grid_res;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    unsigned char *ws = (unsigned char *)workspace;
    int32_t *fine = (int32_t *)ws;
    ws += al(pts * sizeof(int32_t));
    int32_t *rb = (int32_t *)ws;
    ws += al(pts * PSF_MAX_BINS * sizeof(int32_t));
    double *rw = (double *)ws;
    ws += al(pts * PSF_MAX_BINS * sizeof(double));
    unsigned long long *acc = (unsigned long long *)ws;
    ws += al((size_t)total_bins * total_bins * 8);
    double *kw = (double *)ws;
    ws += al((2 * (size_t)radius + 1) * sizeof(double));
    int *flag = (int *)ws;
    SMX_TRY_CUDA(cudaMemcpyAsync(kw, kernel_weights, (2 * (size_t)radius + 1) * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SMX_TRY_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    SMX_TRY_CUDA(cudaMemsetAsync(acc, 0, (size_t)total_bins * total_bins * 8, s));
    fine_bins_kernel<<<blocks_for(pts, 256), 256, 0, s>>>(grid_res, X_lo, X_hi, Y_lo, Y_hi, nX, nY, bin_mapping, fine);
    count_launch();
    psf_rows_kernel<<<blocks_for(pts, 128), 128, 0, s>>>(grid_res, radius, kw, fine, rb, rw, flag);
    count_launch();
    psf_cols_kernel<<<blocks_for(pts, 256), 256, 0, s>>>(grid_res, radius, kw, fine, rb, rw, total_bins, acc);
    count_launch();
    psf_normalise_kernel<<<total_bins, 256, 0, s>>>(acc, total_bins, P);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    int hflag = 0;
    SMX_TRY_CUDA(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (hflag)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_psf_transfer: more than %d bins within the PSF radius of one row",
                         PSF_MAX_BINS);
    return SMX_OK;
}

// ---------------------------------------------------------------- MCMC (RMH)
namespace smx {

// Random-walk Metropolis-Hastings proposal of every chain (the additive normal
// random walk of the reference's sampler, example/example_schwarmax.ipynb cell 12):
//   x' = x + L eps  (L lower triangular, row-major D x D), and the uniform prior's
//   log density: -sum log(hi - lo) inside the box, -inf outside.
__global__ void rmh_propose_kernel(const double *__restrict__ x, const double *__restrict__ L,
                                   const double *__restrict__ eps, int C, int D, const double *__restrict__ lo,
                                   const double *__restrict__ hi, double log_vol, double *xp, double *logprior) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    bool in = true;
    for (int i = 0; i < D; ++i) {
        double s = x[c * D + i];
        for (int j = 0; j <= i; ++j) s += L[i * D + j] * eps[c * D + j];
        xp[c * D + i] = s;
        in = in && (s >= lo[i]) && (s <= hi[i]);
    }
    logprior[c] = in ? -log_vol : -INFINITY;
}

// Metropolis acceptance with the symmetric proposal: accept with probability
// min(1, exp(lp' - lp)) (u < p), the log-likelihood of a proposal replaced by -1e30
// when it is not finite (as the reference's logdensity_fn does).
__global__ void rmh_accept_kernel(double *x, double *lp, const double *__restrict__ xp,
                                  const double *__restrict__ logprior_p, const double *__restrict__ ll_p,
                                  const double *__restrict__ u, int C, int D, int32_t *accepted) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const double ll = ll_p[c];
    const double lpn = logprior_p[c] + (isfinite(ll) ? ll : -1e30);
    const double d = lpn - lp[c];
    const double p = d >= 0 ? 1.0 : exp(d);
    const bool acc = u[c] < p;
    if (acc) {
        for (int i = 0; i < D; ++i) x[c * D + i] = xp[c * D + i];
        lp[c] = lpn;
    }
    accepted[c] = acc ? 1 : 0;
}

}  // namespace smx

extern "C" int smx_rmh_propose(const double *x, const double *L, const double *eps, int n_chains, int ndim,
                               const double *lo, const double *hi, double log_vol, double *x_prop, double *logprior,
                               void *stream) {
    if (n_chains < 1 || ndim < 1 || !x || !L || !eps || !lo || !hi || !x_prop || !logprior)
        return set_error(SMX_ERR_ARGUMENT, "smx_rmh_propose: bad arguments");
    rmh_propose_kernel<<<blocks_for(n_chains, 64), 64, 0, (cudaStream_t)stream>>>(x, L, eps, n_chains, ndim, lo, hi,
                                                                                 log_vol, x_prop, logprior);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

extern "C" int smx_rmh_accept(double *x, double *logdensity, const double *x_prop, const double *logprior_prop,
                              const double *loglike_prop, const double *u, int n_chains, int ndim, int32_t *accepted,
                              void *stream) {
    if (n_chains < 1 || ndim < 1 || !x || !logdensity || !x_prop || !logprior_prop || !loglike_prop || !u || !accepted)
        return set_error(SMX_ERR_ARGUMENT, "smx_rmh_accept: bad arguments");
    rmh_accept_kernel<<<blocks_for(n_chains, 64), 64, 0, (cudaStream_t)stream>>>(x, logdensity, x_prop, logprior_prop,
                                                                                loglike_prop, u, n_chains, ndim,
                                                                                accepted);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}
