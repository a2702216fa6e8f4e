// Projection + binning: stored orbit samples -> one library column per particle.
//
// One CTA per particle.  Its n_real realisations are accumulated into a single
// shared-memory row [Rzphi | xy | h0..h4]; each sample's weight is pre-scaled
// by valid_r / ((sum_r valid_r + 0.1) * T_r), which folds the per-realisation
// normalisation, the validity mask and the realisation mean of
// integrates.py:207-238, 287-298 into the accumulation.  Each thread walks its
// own contiguous stretch of the orbit, so the 32 lanes of a warp sit at
// different orbital phases and rarely hit the same histogram cell in the same
// atomic.  Cell indices follow utils.py:10-42 with explicitly rounded IEEE
// operations (no FMA contraction), in the order
//   norm = (p - lo) / (hi - lo); k = floor(norm * n); clip; oob if norm >= 1 or < 0.
//
// The row is summed in exact fixed point: every term is rounded once to an
// integer multiple of 2^-56 and added as an int64, so the sums do not depend on
// the order of the shared-memory atomics and a library is the same bit for bit
// from run to run.  With the prescaled weights the Rzphi and xy entries of a
// column add up to less than 1, and the h_k terms are accumulated before their
// 1/s_b factor (|g H_k| <= 1 with g = exp(-y^2/2)/sqrt(2 pi)), so every row sum
// stays below 2^6 and the int64 cannot overflow.  The 1/s_b and the xy
// normalisation are applied once per entry when the row is written.
#include "smx_internal.cuh"

namespace smx {

template <typename T> struct RN;
template <> struct RN<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
};
template <> struct RN<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
};

template <typename T> struct GeoT {
    T lo[3], span[3], fn[3];   // Rzphi grid
    int n[3];
    T xlo[2], xspan[2], xfn[2];  // sky grid
    int nx[2];
    T rot[9];
    int n_cells, n_pix, n_bins, rows, n_part, n_real, symmetry;
};

// Returns the flat cell of (a, b, c) or `oob` when any normalised coordinate is
// outside [0, 1).
template <typename T, int D>
__device__ __forceinline__ int grid_cell(const T (&v)[D], const T *lo, const T *span, const T *fn, const int *n,
                                         int oob) {
    int flat = 0, stride = 1;
    bool out = false;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const T norm = RN<T>::div(RN<T>::sub(v[d], lo[d]), span[d]);
        out |= !(norm < T(1)) || norm < T(0);
        int k = (int)floor(RN<T>::mul(norm, fn[d]));
        k = k < 0 ? 0 : (k > n[d] - 1 ? n[d] - 1 : k);
        flat += k * stride;
        stride *= n[d];
    }
    return out ? oob : flat;
}


// Rzphi cell (n_cells = outside), Voronoi bin (-1 = outside) and line-of-sight
// velocity of one phase-space point (integrates.py:120-146).
template <typename T>
__device__ __forceinline__ void project_image(const GeoT<T> &G, const T *rot, T x, T y, T z, T vx, T vy, T vz,
                                              const int32_t *__restrict__ bin_mapping, int &cell, int &b, T &vl) {
    const T R = RN<T>::sqrt(RN<T>::add(RN<T>::mul(x, x), RN<T>::mul(y, y)));
    const T ph = M<T>::atan2(y, x);
    const T cyl[3] = {R, z, ph};
    cell = grid_cell<T, 3>(cyl, G.lo, G.span, G.fn, G.n, G.n_cells);
    const T X = RN<T>::add(RN<T>::add(RN<T>::mul(rot[0], x), RN<T>::mul(rot[1], y)), RN<T>::mul(rot[2], z));
    const T Y = RN<T>::add(RN<T>::add(RN<T>::mul(rot[3], x), RN<T>::mul(rot[4], y)), RN<T>::mul(rot[5], z));
    const T sky[2] = {X, Y};
    const int pix = grid_cell<T, 2>(sky, G.xlo, G.xspan, G.xfn, G.nx, G.n_pix);
    b = __ldg(&bin_mapping[pix]);
    vl = RN<T>::add(RN<T>::add(RN<T>::mul(rot[6], vx), RN<T>::mul(rot[7], vy)), RN<T>::mul(rot[8], vz));
}

// Per-sample cells of the fourfold images, for exactness checks and callers
// that bin on their own: cells/bins (n_img, N) int32, vlos (n_img, N) km/s.
template <typename T>
__global__ void sample_cells_kernel(GeoT<T> G, const T *__restrict__ pts, int64_t N,
                                    const int32_t *__restrict__ bin_mapping, int32_t *cells, int32_t *bins,
                                    T *vlos) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    const T q[6] = {pts[i], pts[N + i], pts[2 * N + i], pts[3 * N + i], pts[4 * N + i], pts[5 * N + i]};
    const int n_img = G.symmetry ? 4 : 1;
    for (int im = 0; im < n_img; ++im) {
        const T sxy = (im >= 2) ? T(-1) : T(1);
        const T sz = (im == 1 || im == 3) ? T(-1) : T(1);
        int cell, b;
        T vl;
        project_image(G, G.rot, sxy * q[0], sxy * q[1], sz * q[2], sxy * q[3], sxy * q[4], sz * q[5], bin_mapping,
                      cell, b, vl);
        cells[im * N + i] = cell;
        bins[im * N + i] = b;
        if (vlos) vlos[im * N + i] = vl * T(kKpcGyrToKms);
    }
}

// round(x 2^56) of a float with |x| < 2^6 as an int64, round half to even (the value of
// __float2ll_rn(x * 2^56)), without the int64 conversion instruction, which runs on the
// FP64 pipe (1/64 of the FP32 rate on this GPU): with t = x 2^24 (exact), t = floor(t) + r,
// r in [0, 1) exact, the result is floor(t) 2^32 + round(r 2^32) (r 2^32 < 2^32).
__device__ __forceinline__ long long fixed56(float x) {
    const float t = x * 0x1p24f;
    const float f = floorf(t);
    const float r = t - f;
    return (long long)(int)f * 4294967296LL + (long long)__float2uint_rn(r * 0x1p32f);
}

// A finite double rounded to the nearest float (ties to even), from its bits; values
// below the normal float range become a signed zero.  Integer operations only (the
// conversion instruction, like all FP64 work, runs at 1/64 of the FP32 rate here).
__device__ __forceinline__ float float_of(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    unsigned long long mant = (b & ((1ull << 52) - 1)) >> 29;
    const unsigned long long rem = b & ((1ull << 29) - 1), half = 1ull << 28;
    mant += (rem > half || (rem == half && (mant & 1))) ? 1 : 0;
    if (mant >> 23) {
        mant = 0;
        ++e;
    }
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)mant);
}

// Adds x rounded to a multiple of 2^-56 (|x| < 2^6) to an int64 fixed-point sum.
__device__ __forceinline__ void fixed_add(unsigned long long *a, float x) {
    atomicAdd(a, (unsigned long long)fixed56(x));
}
__device__ __forceinline__ void fixed_add(unsigned long long *a, double x) {
    atomicAdd(a, (unsigned long long)__double2ll_rn(x * 0x1p56));
}

template <typename T>
__global__ void __launch_bounds__(256) project_bin_kernel(GeoT<T> G, const T *__restrict__ samples,
                                                         const int32_t *__restrict__ n_stored, int64_t slots,
                                                         const T *__restrict__ info, const T *__restrict__ t_total,
                                                         const int32_t *__restrict__ bin_mapping,
                                                         const double *__restrict__ num_per_bin,
                                                         const double *__restrict__ v0g,
                                                         const double *__restrict__ sg, double area_pixel,
                                                         const double *__restrict__ rots, T *library,
                                                         int8_t *valid_out) {
    // batched calls (rots != NULL): CTA b is particle b % n_part of parameter point
    // b / n_part, whose rotation is rots[9 point .. 9 point + 8]; the orbits of all
    // points are numbered consecutively, as smx_integrate_batch stores them
    extern __shared__ unsigned char smem_raw[];
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(smem_raw);
    __shared__ double scale_r[8];
    __shared__ T rot[9];
    const int p = blockIdx.x;   // particle over all points
    const int n_real = G.n_real;
    const int64_t n_orb = (int64_t)G.n_part * n_real * (rots ? (int64_t)gridDim.x / G.n_part : 1);
    if (threadIdx.x < 9) rot[threadIdx.x] = rots ? T(rots[(p / G.n_part) * 9 + threadIdx.x]) : G.rot[threadIdx.x];
    for (int i = threadIdx.x; i < G.rows; i += blockDim.x) acc[i] = 0ull;
    if (threadIdx.x == 0) {
        double v[8];
        double nv = 0;
        for (int r = 0; r < n_real; ++r) {
            const int64_t o = (int64_t)p * n_real + r;
            const double EJ0 = (double)info[SMX_INFO_EJ0 * n_orb + o];
            const double EJ = (double)info[SMX_INFO_EJ * n_orb + o];
            const double tf = (double)info[SMX_INFO_T * n_orb + o];
            // evaluated in the working precision, as |EJ/EJ0 - 1| < 0.1 and t > T/10
            const T dE = M<T>::abs(T(EJ) / T(EJ0) - T(1));
            const bool ok = (dE < T(0.1)) && (T(tf) > t_total[o] / T(10));
            v[r] = ok ? 1.0 : 0.0;
            nv += v[r];
            if (valid_out) valid_out[o] = ok ? 1 : 0;
        }
        for (int r = 0; r < n_real; ++r) {
            const int64_t o = (int64_t)p * n_real + r;
            const double wsum = (double)info[SMX_INFO_WSUM * n_orb + o];
            const double Ti = (G.symmetry ? 4.0 : 1.0) * wsum + kEps;
            scale_r[r] = v[r] / ((nv + 0.1) * Ti);
        }
    }
    __syncthreads();
    const int off_xy = G.n_cells;
    const int off_h = G.n_cells + G.n_bins;
    const int nb = G.n_bins;
    const T kms = T(kKpcGyrToKms);
    const T isq2pi = T(0.3989422804014327);
    const T sq2 = T(1.4142135623730951), sq3 = T(1.7320508075688772), isq2 = T(0.7071067811865476),
            isq3 = T(0.5773502691896258);
    const int n_img = G.symmetry ? 4 : 1;
    for (int r = 0; r < n_real; ++r) {
        const double scd = scale_r[r];
        if (scd == 0.0) continue;
        const T sc = T(scd);
        const int64_t o = (int64_t)p * n_real + r;
        const int64_t S = n_stored[o];
        const int64_t lo_j = S * threadIdx.x / blockDim.x;
        const int64_t hi_j = S * (threadIdx.x + 1) / blockDim.x;
        const T *base = samples + o * slots;
        const int64_t cs = n_orb * slots;
        for (int64_t j = lo_j; j < hi_j; ++j) {
            const T wraw = base[6 * cs + j];
            if (wraw == T(0)) continue;   // rejected attempts carry no weight
            const T w = wraw * sc;
            const T q[6] = {base[j], base[cs + j], base[2 * cs + j], base[3 * cs + j], base[4 * cs + j], base[5 * cs + j]};
            for (int im = 0; im < n_img; ++im) {
                // sign patterns of integrates.py:74-79
                const T sxy = (im >= 2) ? T(-1) : T(1);
                const T sz = (im == 1 || im == 3) ? T(-1) : T(1);
                const T x = sxy * q[0], y = sxy * q[1], z = sz * q[2];
                const T vx = sxy * q[3], vy = sxy * q[4], vz = sz * q[5];
                int cell, b;
                T vl;
                project_image(G, rot, x, y, z, vx, vy, vz, bin_mapping, cell, b, vl);
                if (cell < G.n_cells) fixed_add(&acc[cell], w);
                if (b < 0 || b >= nb) continue;
                T s_b, v0_b;
                if constexpr (sizeof(T) == 4) {
                    s_b = float_of(__ldg(&sg[b]));
                    v0_b = float_of(__ldg(&v0g[b]));
                } else {
                    s_b = __ldg(&sg[b]);
                    v0_b = __ldg(&v0g[b]);
                }
                const T yv = (vl * kms - v0_b) / s_b;
                // g without its 1/s_b (applied when the row is written)
                const T gw = w * isq2pi * M<T>::exp(T(-0.5) * yv * yv);
                const T H1 = sq2 * yv;
                const T H2 = (sq2 * yv * H1 - T(1)) * isq2;
                const T H3 = (sq2 * yv * H2 - sq2 * H1) * isq3;
                const T H4 = (sq2 * yv * H3 - sq3 * H2) * T(0.5);
                fixed_add(&acc[off_xy + b], w);
                fixed_add(&acc[off_h + b], gw);
                fixed_add(&acc[off_h + nb + b], gw * H1);
                fixed_add(&acc[off_h + 2 * nb + b], gw * H2);
                fixed_add(&acc[off_h + 3 * nb + b], gw * H3);
                fixed_add(&acc[off_h + 4 * nb + b], gw * H4);
            }
        }
    }
    __syncthreads();
    T *col = library + (int64_t)p * G.rows;
    if (sizeof(T) == 4) {
        // float library: the entry and its normalisation in float (a product with the
        // rounded reciprocal, within 1.5 float ulp of the quotient), so that the FP64
        // pipe, 1/64 of the FP32 rate here, does no division per entry
        for (int i = threadIdx.x; i < G.rows; i += blockDim.x) {
            float v = (float)(long long)acc[i] * 0x1p-56f;
            if (i >= off_xy && i < off_h) v *= 1.0f / (float)(num_per_bin[i - off_xy] * area_pixel + kEps);
            else if (i >= off_h) v *= 1.0f / (float)sg[(i - off_h) % nb];
            col[i] = T(v);
        }
    } else {
        for (int i = threadIdx.x; i < G.rows; i += blockDim.x) {
            double v = (double)(long long)acc[i] * 0x1p-56;
            if (i >= off_xy && i < off_h) v = v / (num_per_bin[i - off_xy] * area_pixel + kEps);
            else if (i >= off_h) v = v / sg[(i - off_h) % nb];
            col[i] = T(v);
        }
    }
}

template <typename T>
static GeoT<T> make_geo(const smx_binning *g) {
    GeoT<T> G;
    const double lo[3] = {g->R_lo, g->z_lo, g->phi_lo}, hi[3] = {g->R_hi, g->z_hi, g->phi_hi};
    const int n[3] = {g->nR, g->nz, g->nphi};
    for (int d = 0; d < 3; ++d) {
        G.lo[d] = T(lo[d]);
        G.span[d] = T(hi[d]) - T(lo[d]);
        G.fn[d] = T(n[d]);
        G.n[d] = n[d];
    }
    const double xlo[2] = {g->X_lo, g->Y_lo}, xhi[2] = {g->X_hi, g->Y_hi};
    const int nx[2] = {g->nX, g->nY};
    for (int d = 0; d < 2; ++d) {
        G.xlo[d] = T(xlo[d]);
        G.xspan[d] = T(xhi[d]) - T(xlo[d]);
        G.xfn[d] = T(nx[d]);
        G.nx[d] = nx[d];
    }
    for (int i = 0; i < 9; ++i) G.rot[i] = T(g->rot[i]);
    G.n_cells = g->nR * g->nz * g->nphi;
    G.n_pix = g->nX * g->nY;
    G.n_bins = g->n_bins;
    G.rows = G.n_cells + 6 * g->n_bins;
    G.n_part = g->n_part;
    G.n_real = g->n_real;
    G.symmetry = g->symmetry;
    return G;
}

template <typename T>
static int launch(const smx_binning *g, const void *samples, const int32_t *n_stored, int64_t slots,
                  const void *info, const void *t_total, const int32_t *bin_mapping, const double *num_per_bin,
                  const double *v0, const double *s, void *library, int8_t *valid, cudaStream_t st,
                  const double *rots = nullptr, int n_points = 1) {
    const GeoT<T> G = make_geo<T>(g);
    const size_t smem = (size_t)G.rows * sizeof(unsigned long long);
    int dev = 0, max_smem = 0;
    SMX_TRY_CUDA(cudaGetDevice(&dev));
    SMX_TRY_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem + 1024 > (size_t)max_smem)
        return set_error(SMX_ERR_UNSUPPORTED, "library row of %d entries does not fit in shared memory", G.rows);
    SMX_TRY_CUDA(cudaFuncSetAttribute(project_bin_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const double area = ((g->X_hi - g->X_lo) / g->nX) * ((g->Y_hi - g->Y_lo) / g->nY) * 1e6;
    const int64_t ctas = (int64_t)g->n_part * n_points;
    if (ctas > 0x7fffffffLL) return set_error(SMX_ERR_UNSUPPORTED, "smx_project_bin: too many particles");
    project_bin_kernel<T><<<(unsigned)ctas, 256, smem, st>>>(G, (const T *)samples, n_stored, slots, (const T *)info,
                                                             (const T *)t_total, bin_mapping, num_per_bin, v0, s, area,
                                                             rots, (T *)library, valid);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

}  // namespace smx

using namespace smx;

extern "C" int smx_project_bin(const smx_binning *geo, int precision, const void *samples, const int32_t *n_stored,
                               int64_t slots, const void *info, const void *t_total, const int32_t *bin_mapping,
                               const double *num_per_bin, const double *v0, const double *s, void *library,
                               int8_t *valid, void *stream) {
    if (!geo) return set_error(SMX_ERR_ARGUMENT, "smx_project_bin: geometry is NULL");
    if (geo->n_part < 0 || geo->n_real < 1 || geo->n_real > 8 || geo->nR < 1 || geo->nz < 1 || geo->nphi < 1 ||
        geo->nX < 1 || geo->nY < 1 || geo->n_bins < 1 || slots < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_project_bin: bad sizes (n_real must be 1..8)");
    if (!(geo->R_hi > geo->R_lo) || !(geo->z_hi > geo->z_lo) || !(geo->phi_hi > geo->phi_lo) ||
        !(geo->X_hi > geo->X_lo) || !(geo->Y_hi > geo->Y_lo))
        return set_error(SMX_ERR_ARGUMENT, "smx_project_bin: empty grid range");
    if (geo->n_part == 0) return SMX_OK;
    if (!samples || !n_stored || !info || !t_total || !bin_mapping || !num_per_bin || !v0 || !s || !library)
        return set_error(SMX_ERR_ARGUMENT, "smx_project_bin: NULL buffer");
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == SMX_FP32)
        return launch<float>(geo, samples, n_stored, slots, info, t_total, bin_mapping, num_per_bin, v0, s, library,
                             valid, st);
    if (precision == SMX_FP64)
        return launch<double>(geo, samples, n_stored, slots, info, t_total, bin_mapping, num_per_bin, v0, s, library,
                              valid, st);
    return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
}

extern "C" int smx_project_bin_batch(const smx_binning *geo, int n_points, const double *rots, int precision,
                                     const void *samples, const int32_t *n_stored, int64_t slots, const void *info,
                                     const void *t_total, const int32_t *bin_mapping, const double *num_per_bin,
                                     const double *v0, const double *s, void *library, int8_t *valid, void *stream) {
    if (!geo || !rots) return set_error(SMX_ERR_ARGUMENT, "smx_project_bin_batch: geometry or rotations NULL");
    if (n_points < 1) return set_error(SMX_ERR_ARGUMENT, "smx_project_bin_batch: n_points < 1");
    if (geo->n_part < 0 || geo->n_real < 1 || geo->n_real > 8 || geo->nR < 1 || geo->nz < 1 || geo->nphi < 1 ||
        geo->nX < 1 || geo->nY < 1 || geo->n_bins < 1 || slots < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_project_bin_batch: bad sizes (n_real must be 1..8)");
    if (!(geo->R_hi > geo->R_lo) || !(geo->z_hi > geo->z_lo) || !(geo->phi_hi > geo->phi_lo) ||
        !(geo->X_hi > geo->X_lo) || !(geo->Y_hi > geo->Y_lo))
        return set_error(SMX_ERR_ARGUMENT, "smx_project_bin_batch: empty grid range");
    if (geo->n_part == 0) return SMX_OK;
    if (!samples || !n_stored || !info || !t_total || !bin_mapping || !num_per_bin || !v0 || !s || !library)
        return set_error(SMX_ERR_ARGUMENT, "smx_project_bin_batch: NULL buffer");
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == SMX_FP32)
        return launch<float>(geo, samples, n_stored, slots, info, t_total, bin_mapping, num_per_bin, v0, s, library,
                             valid, st, rots, n_points);
    if (precision == SMX_FP64)
        return launch<double>(geo, samples, n_stored, slots, info, t_total, bin_mapping, num_per_bin, v0, s, library,
                              valid, st, rots, n_points);
    return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
}

extern "C" int smx_sample_cells(const smx_binning *geo, int precision, const void *points, int64_t n,
                                const int32_t *bin_mapping, int32_t *cells, int32_t *bins, void *vlos,
                                void *stream) {
    if (!geo) return set_error(SMX_ERR_ARGUMENT, "smx_sample_cells: geometry is NULL");
    if (n < 0 || geo->nR < 1 || geo->nz < 1 || geo->nphi < 1 || geo->nX < 1 || geo->nY < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_sample_cells: bad sizes");
    if (n == 0) return SMX_OK;
    if (!points || !bin_mapping || !cells || !bins) return set_error(SMX_ERR_ARGUMENT, "smx_sample_cells: NULL buffer");
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (precision == SMX_FP32) {
        sample_cells_kernel<float><<<grid, 256, 0, st>>>(make_geo<float>(geo), (const float *)points, n, bin_mapping,
                                                         cells, bins, (float *)vlos);
        count_launch();
    } else if (precision == SMX_FP64) {
        sample_cells_kernel<double><<<grid, 256, 0, st>>>(make_geo<double>(geo), (const double *)points, n,
                                                          bin_mapping, cells, bins, (double *)vlos);
        count_launch();
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}
