// Differentiable projection (no reference counterpart; the reference stops
// gradients at its NNLS, nnls.py:66,165): the sky rows [xy | h0..h4] of the
// library with soft aperture assignment, and their adjoint with respect to the
// viewing angles (alpha, beta, gamma) and a line-of-sight velocity scale.
//
// Each sample image at sky position (X, Y) (pixel coordinates u, v) is spread
// over the pixels by a Gaussian of width sigma (pixels), integrated over each
// pixel:  w_ij = wx_i(u) wy_j(v),  wx_i(u) = [erf((i + 1 - u)/(sqrt2 sigma)) -
// erf((i - u)/(sqrt2 sigma))] / 2, over a window of +-3 pixels (at sigma = 0.5
// pixel the mass outside it is below 1e-6).  The weights of the pixels of one
// Voronoi bin are summed, W_b, and the sample adds, like the hard binning of
// integrates.py:115-174,
//   xy_b += w W_b,   h_k,b += w W_b g(y_b) H_k(y_b),   y_b = (s_v v_los - v0_b)/s_b,
// with the same per-realisation normalisation and validity as smx_project_bin.
// The adjoint recomputes every rotated sample (nothing is stored) and reduces
//   dL/dtheta = sum over samples of  w sum_b [c_xy,b dW_b/dtheta + sum_k c_hk,b d(W_b g H_k)/dtheta]
// with dW_b/dtheta from dwx/du du/dtheta and dwy/dv dv/dtheta, and
// d(g H_k)/dy = g (sqrt(2k) H_{k-1} - y H_k).
#include "smx_internal.cuh"

namespace smx {

namespace soft {

constexpr int WIN = 3;                  // window half-width in pixels
constexpr int NW = 2 * WIN + 1;
constexpr int MAXB = 12;                // distinct bins merged per sample image

template <typename T> struct Geo {
    T xlo, ylo, dx, dy;                 // sky grid
    int nX, nY, n_bins, n_cells, rows, n_part, n_real, symmetry;
    T rot[9];                           // rows: X, Y, line of sight
    T drot[3][9];                       // d rot / d alpha, beta, gamma
    T isig;                             // 1 / (sqrt2 sigma)
    T dnorm;                            // 1 / (sqrt(2 pi) sigma)
    T vscale;
};

template <typename T>
__device__ __forceinline__ T erf_(T x) { return sizeof(T) == 8 ? (T)erf((double)x) : (T)erff((float)x); }

// pixel weights of one coordinate (pixel units) and their derivatives; first = first pixel of the window
template <typename T>
__device__ __forceinline__ void axis_weights(T u, int n, T isig, T dnorm, T (&w)[NW], T (&dw)[NW], int &first) {
    // far outside the grid every weight is 0; the clamp keeps the integer conversion in range
    u = u < T(-16) ? T(-16) : (u > T(n + 16) ? T(n + 16) : u);
    first = (int)floor(u) - WIN;
    T e_lo = erf_((T(first) - u) * isig);
    T g_lo = exp(-((T(first) - u) * isig) * ((T(first) - u) * isig));
#pragma unroll
    for (int k = 0; k < NW; ++k) {
        const T t = (T(first + k + 1) - u) * isig;
        const T e_hi = erf_(t);
        const T g_hi = exp(-t * t);
        const bool in = (first + k) >= 0 && (first + k) < n;
        w[k] = in ? T(0.5) * (e_hi - e_lo) : T(0);
        dw[k] = in ? dnorm * (g_lo - g_hi) : T(0);   // d w / d u
        e_lo = e_hi;
        g_lo = g_hi;
    }
}

struct SoftArgs {
    const void *samples;
    const int32_t *n_stored;
    int64_t slots;
    const void *info, *t_total;
    const int32_t *bin_mapping;
    const double *num_per_bin, *v0, *s;
    double area;
};

// per-realisation sample scale (validity and normalisation of smx_project_bin)
template <typename T>
__device__ void realisation_scales(const Geo<T> &G, const SoftArgs &a, int p, double *scale_r) {
    const T *info = (const T *)a.info;
    const T *t_total = (const T *)a.t_total;
    const int64_t n_orb = (int64_t)G.n_part * G.n_real;
    double v[8];
    double nv = 0;
    for (int r = 0; r < G.n_real; ++r) {
        const int64_t o = (int64_t)p * G.n_real + r;
        const T dE = M<T>::abs(info[SMX_INFO_EJ * n_orb + o] / info[SMX_INFO_EJ0 * n_orb + o] - T(1));
        const bool ok = (dE < T(0.1)) && (info[SMX_INFO_T * n_orb + o] > t_total[o] / T(10));
        v[r] = ok ? 1.0 : 0.0;
        nv += v[r];
    }
    for (int r = 0; r < G.n_real; ++r) {
        const int64_t o = (int64_t)p * G.n_real + r;
        const double Ti = (G.symmetry ? 4.0 : 1.0) * (double)info[SMX_INFO_WSUM * n_orb + o] + kEps;
        scale_r[r] = v[r] / ((nv + 0.1) * Ti);
    }
}

// one sample image: calls f(bin, W, dW/du, dW/dv) for every Voronoi bin its
// window touches, with the pixel weights of the bin summed.  Up to MAXB bins are
// merged; a pixel of a further bin is passed on its own (the contributions are
// linear in the pixel weights, so the result is the same).
template <typename T, typename F>
__device__ __forceinline__ void for_bins(const Geo<T> &G, const int32_t *__restrict__ bin_mapping, T u, T v, F &&f) {
    T wx[NW], dwx[NW], wy[NW], dwy[NW];
    int fx, fy;
    axis_weights(u, G.nX, G.isig, G.dnorm, wx, dwx, fx);
    axis_weights(v, G.nY, G.isig, G.dnorm, wy, dwy, fy);
    int bins[MAXB];
    T W[MAXB], Wu[MAXB], Wv[MAXB];
    int nb = 0;
    for (int j = 0; j < NW; ++j) {
        if (wy[j] == T(0) && dwy[j] == T(0)) continue;
        for (int i = 0; i < NW; ++i) {
            if (wx[i] == T(0) && dwx[i] == T(0)) continue;
            const int b = __ldg(&bin_mapping[(fx + i) + G.nX * (fy + j)]);
            if (b < 0 || b >= G.n_bins) continue;
            int slot = -1;
            for (int q = 0; q < nb; ++q)
                if (bins[q] == b) slot = q;
            if (slot < 0) {
                if (nb == MAXB) {
                    f(b, wx[i] * wy[j], dwx[i] * wy[j], wx[i] * dwy[j]);
                    continue;
                }
                slot = nb++;
                bins[slot] = b;
                W[slot] = Wu[slot] = Wv[slot] = T(0);
            }
            W[slot] += wx[i] * wy[j];
            Wu[slot] += dwx[i] * wy[j];
            Wv[slot] += wx[i] * dwy[j];
        }
    }
    for (int q = 0; q < nb; ++q) f(bins[q], W[q], Wu[q], Wv[q]);
}

template <typename T>
__device__ __forceinline__ void hermite(T y, T (&H)[5]) {
    const T sq2 = T(1.4142135623730951), sq3 = T(1.7320508075688772);
    H[0] = T(1);
    H[1] = sq2 * y;
    H[2] = (sq2 * y * H[1] - T(1)) * T(0.7071067811865476);
    H[3] = (sq2 * y * H[2] - sq2 * H[1]) * T(0.5773502691896258);
    H[4] = (sq2 * y * H[3] - sq3 * H[2]) * T(0.5);
}

// forward: one CTA per particle, the sky rows of the library accumulated with
// global reductions (red_add).  In double they are exact int64 fixed-point sums
// in units of 2^-56 (every row sum stays below 64), stored in place of the
// doubles and converted after, so the rows do not depend on the order of the
// adds.  Float rows take float adds.  Separate kernels zero the rows before and
// convert / normalise them after.
__device__ __forceinline__ void add(float *p, float v) { red_add(p, v); }
__device__ __forceinline__ void add(double *p, double v) {
    red_add(reinterpret_cast<unsigned long long *>(p), (unsigned long long)__double2ll_rn(v * 0x1p56));
}

template <typename T>
__global__ void __launch_bounds__(256, 1) soft_project_kernel(Geo<T> G, SoftArgs a, T *library) {
    __shared__ double scale_r[8];
    const int p = blockIdx.x;
    const int nbins = G.n_bins;
    if (threadIdx.x == 0) realisation_scales(G, a, p, scale_r);
    __syncthreads();
    T *acc = library + (int64_t)p * G.rows + G.n_cells;   // [xy | h0..h4] of this particle
    const T *samples = (const T *)a.samples;
    const int64_t n_orb = (int64_t)G.n_part * G.n_real;
    const int64_t cs = n_orb * a.slots;
    const T kms = T(kKpcGyrToKms), isq2pi = T(0.3989422804014327);
    const int n_img = G.symmetry ? 4 : 1;
    for (int r = 0; r < G.n_real; ++r) {
        if (scale_r[r] == 0.0) continue;
        const T sc = T(scale_r[r]);
        const int64_t o = (int64_t)p * G.n_real + r;
        const int64_t S = a.n_stored[o];
        const T *base = samples + o * a.slots;
        // each thread walks its own contiguous stretch of the orbit, so the lanes of a
        // warp sit at different phases and rarely add to the same bin at once
        const int64_t lo_j = S * threadIdx.x / blockDim.x, hi_j = S * (threadIdx.x + 1) / blockDim.x;
        for (int64_t j = lo_j; j < hi_j; ++j) {
            const T wraw = base[6 * cs + j];
            if (wraw == T(0)) continue;
            const T w = wraw * sc;
            const T q[6] = {base[j], base[cs + j], base[2 * cs + j], base[3 * cs + j], base[4 * cs + j], base[5 * cs + j]};
            for (int im = 0; im < n_img; ++im) {
                const T sxy = (im >= 2) ? T(-1) : T(1);
                const T sz = (im == 1 || im == 3) ? T(-1) : T(1);
                const T x = sxy * q[0], y = sxy * q[1], z = sz * q[2];
                const T vx = sxy * q[3], vy = sxy * q[4], vz = sz * q[5];
                const T X = G.rot[0] * x + G.rot[1] * y + G.rot[2] * z;
                const T Y = G.rot[3] * x + G.rot[4] * y + G.rot[5] * z;
                const T vl = G.vscale * (G.rot[6] * vx + G.rot[7] * vy + G.rot[8] * vz) * kms;
                for_bins(G, a.bin_mapping, (X - G.xlo) / G.dx, (Y - G.ylo) / G.dy, [&](int b, T Wb, T, T) {
                    const T sb = T(__ldg(&a.s[b]));
                    const T yv = (vl - T(__ldg(&a.v0[b]))) / sb;
                    const T gw = w * Wb * isq2pi / sb * exp(T(-0.5) * yv * yv);
                    T H[5];
                    hermite(yv, H);
                    add(&acc[b], w * Wb);
#pragma unroll
                    for (int k = 0; k < 5; ++k) add(&acc[(1 + k) * nbins + b], gw * H[k]);
                });
            }
        }
    }
}

// sky rows of every particle: zero (mode 0), or (mode 1) convert the fixed-point
// sums of double rows and divide the xy row by num_per_bin x area
template <typename T>
__global__ void sky_rows_kernel(T *library, int64_t n_part, int rows, int n_cells, int nbins,
                                const double *__restrict__ num_per_bin, double area, int mode) {
    const int64_t per = 6 * (int64_t)nbins;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_part * per;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = k / per, i = k % per;
        T *v = library + p * rows + n_cells + i;
        if (mode == 0) {
            *v = T(0);   // also int64 0 in double rows
        } else {
            double x = (double)*v;
            if (sizeof(T) == 8) x = (double)*reinterpret_cast<const long long *>(v) * 0x1p-56;
            if (i < nbins) x /= num_per_bin[i] * area + kEps;
            *v = T(x);
        }
    }
}

// adjoint: one CTA per particle; cot (n_part, rows) cotangent of the library
// (only the sky rows are read); grad[0..3] += dL/d(alpha, beta, gamma, vscale)
template <typename T>
__global__ void __launch_bounds__(256) soft_adjoint_kernel(Geo<T> G, SoftArgs a, const T *__restrict__ cot,
                                                          double *grad) {
    extern __shared__ unsigned char smem_raw[];
    T *c = reinterpret_cast<T *>(smem_raw);   // 6 n_bins cotangents (xy already divided by its normalisation)
    __shared__ double scale_r[8];
    __shared__ double red[8][4];
    const int p = blockIdx.x;
    const int nbins = G.n_bins;
    const T *crow = cot + (int64_t)p * G.rows + G.n_cells;
    for (int i = threadIdx.x; i < 6 * nbins; i += blockDim.x) {
        T v = crow[i];
        if (i < nbins) v = T((double)v / (a.num_per_bin[i] * a.area + kEps));
        c[i] = v;
    }
    if (threadIdx.x == 0) realisation_scales(G, a, p, scale_r);
    __syncthreads();
    const T *samples = (const T *)a.samples;
    const int64_t n_orb = (int64_t)G.n_part * G.n_real;
    const int64_t cs = n_orb * a.slots;
    const T kms = T(kKpcGyrToKms), isq2pi = T(0.3989422804014327);
    const T sqk[5] = {T(0), T(1.4142135623730951), T(2), T(2.449489742783178), T(2.8284271247461903)};
    const int n_img = G.symmetry ? 4 : 1;
    double gacc[4] = {0, 0, 0, 0};
    for (int r = 0; r < G.n_real; ++r) {
        if (scale_r[r] == 0.0) continue;
        const T sc = T(scale_r[r]);
        const int64_t o = (int64_t)p * G.n_real + r;
        const int64_t S = a.n_stored[o];
        const T *base = samples + o * a.slots;
        for (int64_t j = threadIdx.x; j < S; j += blockDim.x) {
            const T wraw = base[6 * cs + j];
            if (wraw == T(0)) continue;
            const T w = wraw * sc;
            const T q[6] = {base[j], base[cs + j], base[2 * cs + j], base[3 * cs + j], base[4 * cs + j], base[5 * cs + j]};
            for (int im = 0; im < n_img; ++im) {
                const T sxy = (im >= 2) ? T(-1) : T(1);
                const T sz = (im == 1 || im == 3) ? T(-1) : T(1);
                const T x = sxy * q[0], y = sxy * q[1], z = sz * q[2];
                const T vx = sxy * q[3], vy = sxy * q[4], vz = sz * q[5];
                const T X = G.rot[0] * x + G.rot[1] * y + G.rot[2] * z;
                const T Y = G.rot[3] * x + G.rot[4] * y + G.rot[5] * z;
                const T vraw = (G.rot[6] * vx + G.rot[7] * vy + G.rot[8] * vz) * kms;
                const T vl = G.vscale * vraw;
                // derivatives of u, v and v_los with respect to alpha, beta, gamma, vscale
                T du[4], dv[4], dvl[4];
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    du[t] = (G.drot[t][0] * x + G.drot[t][1] * y + G.drot[t][2] * z) / G.dx;
                    dv[t] = (G.drot[t][3] * x + G.drot[t][4] * y + G.drot[t][5] * z) / G.dy;
                    dvl[t] = G.vscale * (G.drot[t][6] * vx + G.drot[t][7] * vy + G.drot[t][8] * vz) * kms;
                }
                du[3] = dv[3] = T(0);
                dvl[3] = vraw;
                for_bins(G, a.bin_mapping, (X - G.xlo) / G.dx, (Y - G.ylo) / G.dy, [&](int b, T Wb, T Wu, T Wv) {
                    const T sb = T(__ldg(&a.s[b]));
                    const T yv = (vl - T(__ldg(&a.v0[b]))) / sb;
                    const T g = isq2pi / sb * exp(T(-0.5) * yv * yv);
                    T H[5];
                    hermite(yv, H);
                    // A = c_xy + sum_k c_hk g H_k (coefficient of W_b), Bd = sum_k c_hk d(g H_k)/dy
                    T A = c[b], Bd = T(0);
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        const T ck = c[(1 + k) * nbins + b];
                        A += ck * g * H[k];
                        Bd += ck * g * ((k > 0 ? sqk[k] * H[k - 1] : T(0)) - yv * H[k]);
                    }
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const T dW = Wu * du[t] + Wv * dv[t];
                        gacc[t] += (double)(w * (A * dW + Wb * Bd * dvl[t] / sb));
                    }
                });
            }
        }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        double v = gacc[t];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
        atomicAdd(&grad[threadIdx.x], v);
    }
}

template <typename T>
static Geo<T> make(const smx_binning *g, double sigma_pix, double vscale, const double *drot) {
    Geo<T> G;
    G.xlo = T(g->X_lo);
    G.ylo = T(g->Y_lo);
    G.dx = T((g->X_hi - g->X_lo) / g->nX);
    G.dy = T((g->Y_hi - g->Y_lo) / g->nY);
    G.nX = g->nX;
    G.nY = g->nY;
    G.n_bins = g->n_bins;
    G.n_cells = g->nR * g->nz * g->nphi;
    G.rows = G.n_cells + 6 * g->n_bins;
    G.n_part = g->n_part;
    G.n_real = g->n_real;
    G.symmetry = g->symmetry;
    for (int i = 0; i < 9; ++i) G.rot[i] = T(g->rot[i]);
    for (int t = 0; t < 3; ++t)
        for (int i = 0; i < 9; ++i) G.drot[t][i] = drot ? T(drot[t * 9 + i]) : T(0);
    G.isig = T(1.0 / (1.4142135623730951 * sigma_pix));
    G.dnorm = T(1.0 / (2.5066282746310002 * sigma_pix));
    G.vscale = T(vscale);
    return G;
}

static int check(const smx_binning *g, double sigma_pix, double vscale, const char *who) {
    if (!g) return set_error(SMX_ERR_ARGUMENT, "%s: geometry is NULL", who);
    if (g->n_part < 0 || g->n_real < 1 || g->n_real > 8 || g->nX < 1 || g->nY < 1 || g->n_bins < 1 || g->nR < 1 ||
        g->nz < 1 || g->nphi < 1)
        return set_error(SMX_ERR_ARGUMENT, "%s: bad sizes (n_real must be 1..8)", who);
    if (!(g->X_hi > g->X_lo) || !(g->Y_hi > g->Y_lo)) return set_error(SMX_ERR_ARGUMENT, "%s: empty sky grid", who);
    if (!(sigma_pix >= 0.05 && sigma_pix <= 1.0))
        return set_error(SMX_ERR_ARGUMENT, "%s: sigma must be in [0.05, 1] pixel (window of +-3 pixels)", who);
    if (!(vscale > 0)) return set_error(SMX_ERR_ARGUMENT, "%s: velocity scale must be > 0", who);
    return SMX_OK;
}

}  // namespace soft

}  // namespace smx

using namespace smx;

extern "C" int smx_soft_project(const smx_binning *geo, int precision, double sigma_pix, double vscale,
                                const void *samples, const int32_t *n_stored, int64_t slots, const void *info,
                                const void *t_total, const int32_t *bin_mapping, const double *num_per_bin,
                                const double *v0, const double *s, void *library, void *stream) {
    int st = soft::check(geo, sigma_pix, vscale, "smx_soft_project");
    if (st) return st;
    if (geo->n_part == 0) return SMX_OK;
    if (!samples || !n_stored || !info || !t_total || !bin_mapping || !num_per_bin || !v0 || !s || !library || slots < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_soft_project: NULL buffer or bad slots");
    soft::SoftArgs a{samples, n_stored, slots, info, t_total, bin_mapping, num_per_bin, v0, s,
                     ((geo->X_hi - geo->X_lo) / geo->nX) * ((geo->Y_hi - geo->Y_lo) / geo->nY) * 1e6};
    cudaStream_t sm = (cudaStream_t)stream;
    const int rows = geo->nR * geo->nz * geo->nphi + 6 * geo->n_bins;
    const int n_cells = geo->nR * geo->nz * geo->nphi;
    const int64_t cnt = (int64_t)geo->n_part * 6 * geo->n_bins;
    const unsigned g1 = (unsigned)((cnt + 255) / 256 < 152 * 64 ? (cnt + 255) / 256 : 152 * 64);
    if (precision == SMX_FP32) {
        soft::sky_rows_kernel<float><<<g1, 256, 0, sm>>>((float *)library, geo->n_part, rows, n_cells, geo->n_bins,
                                                          num_per_bin, a.area, 0);
        soft::soft_project_kernel<float><<<geo->n_part, 256, 0, sm>>>(soft::make<float>(geo, sigma_pix, vscale, nullptr),
                                                                      a, (float *)library);
        soft::sky_rows_kernel<float><<<g1, 256, 0, sm>>>((float *)library, geo->n_part, rows, n_cells, geo->n_bins,
                                                          num_per_bin, a.area, 1);
    } else if (precision == SMX_FP64) {
        soft::sky_rows_kernel<double><<<g1, 256, 0, sm>>>((double *)library, geo->n_part, rows, n_cells, geo->n_bins,
                                                           num_per_bin, a.area, 0);
        soft::soft_project_kernel<double><<<geo->n_part, 256, 0, sm>>>(
            soft::make<double>(geo, sigma_pix, vscale, nullptr), a, (double *)library);
        soft::sky_rows_kernel<double><<<g1, 256, 0, sm>>>((double *)library, geo->n_part, rows, n_cells, geo->n_bins,
                                                           num_per_bin, a.area, 1);
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    count_launch(3);
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

extern "C" int smx_soft_project_adjoint(const smx_binning *geo, int precision, double sigma_pix, double vscale,
                                        const double *drot, const void *samples, const int32_t *n_stored, int64_t slots,
                                        const void *info, const void *t_total, const int32_t *bin_mapping,
                                        const double *num_per_bin, const double *v0, const double *s,
                                        const void *cotangent, double *grad, void *stream) {
    int st = soft::check(geo, sigma_pix, vscale, "smx_soft_project_adjoint");
    if (st) return st;
    if (!drot || !grad) return set_error(SMX_ERR_ARGUMENT, "smx_soft_project_adjoint: NULL drot or grad");
    if (geo->n_part == 0) return SMX_OK;
    if (!samples || !n_stored || !info || !t_total || !bin_mapping || !num_per_bin || !v0 || !s || !cotangent ||
        slots < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_soft_project_adjoint: NULL buffer or bad slots");
    soft::SoftArgs a{samples, n_stored, slots, info, t_total, bin_mapping, num_per_bin, v0, s,
                     ((geo->X_hi - geo->X_lo) / geo->nX) * ((geo->Y_hi - geo->Y_lo) / geo->nY) * 1e6};
    cudaStream_t sm = (cudaStream_t)stream;
    if (precision == SMX_FP32) {
        const size_t smem = (size_t)6 * geo->n_bins * sizeof(float);
        SMX_TRY_CUDA(cudaFuncSetAttribute(soft::soft_adjoint_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        soft::soft_adjoint_kernel<float><<<geo->n_part, 256, smem, sm>>>(soft::make<float>(geo, sigma_pix, vscale, drot),
                                                                         a, (const float *)cotangent, grad);
    } else if (precision == SMX_FP64) {
        const size_t smem = (size_t)6 * geo->n_bins * sizeof(double);
        SMX_TRY_CUDA(cudaFuncSetAttribute(soft::soft_adjoint_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        soft::soft_adjoint_kernel<double><<<geo->n_part, 256, smem, sm>>>(
            soft::make<double>(geo, sigma_pix, vscale, drot), a, (const double *)cotangent, grad);
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}
