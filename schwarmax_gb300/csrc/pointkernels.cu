// Point-wise kernels: potential/force/density evaluation, the fused per-particle
// initial conditions (Jeans velocities + V_c + T_orb + jitter) and the 3-D
// density target.
#include "smx_internal.cuh"

namespace smx {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void potential_eval_kernel(PotT<T> P, const T *__restrict__ x, const T *__restrict__ y,
                                      const T *__restrict__ z, int64_t n, T *phi, T *ax, T *ay, T *az,
                                      T *rho) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T X = x[i], Y = y[i], Z = z[i];
    if (ax || ay || az) {
        T p, gx, gy, gz;
        potential<T, true, true>(P, X, Y, Z, p, gx, gy, gz);
        if (phi) phi[i] = p;
        if (ax) ax[i] = -gx;
        if (ay) ay[i] = -gy;
        if (az) az[i] = -gz;
    } else if (phi) {
        phi[i] = phi_only(P, X, Y, Z);
    }
    if (rho) rho[i] = density(P, X, Y, Z);
}

// One warp per particle.  jeans.py:8-93 with the vertical integrals split over
// the 32 lanes (1000 trapezoid points each), then utils.py:182-273 for V_c and
// T_orb at the new (R, z) and the jitter of model.py:127-148.
// CANON: the bar and bulge slots hold T3 / V4 and there is no spline component (the
// compile-time path of the potential, as in the integrator).
template <typename T, bool CANON>
__global__ void initial_conditions_kernel(PotT<T> P, const T *__restrict__ pos, const T *__restrict__ normals,
                                          const T *__restrict__ unif, int64_t n, int n_real, T n_periods,
                                          T steps_pp, T *w_out, T *t_total, T *dt_init, T *w0_new, T *t_orb,
                                          T *vc) {
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= n) return;   // uniform per warp
    const int64_t p = gw;
    const T x = pos[p], y = pos[n + p], z = pos[2 * n + p];
    const T R = M<T>::sqrt(x * x + y * y);
    const T za = M<T>::abs(z);
    const T ztop = T(10);
    const int NQ = 1000;
    const T dzq = (ztop - za) / T(NQ - 1);
    const T d = T(5e-3);
    const T i2d = T(1) / (T(2) * d);
    const T zero = T(0);
    T s0 = 0, sp = 0, sm = 0;
    for (int j = lane; j < NQ; j += 32) {
        const T zj = (j == NQ - 1) ? ztop : za + T(j) * dzq;
        const T wj = (j == 0 || j == NQ - 1) ? T(0.5) : T(1);
        const T f0 = density(P, x, y, zj) * (phi_only<T, CANON>(P, x, y, zj + d) - phi_only<T, CANON>(P, x, y, zj - d)) * i2d;
        const T Rp = R + d, Rm = R - d;
        const T fp = density(P, Rp, zero, zj) * (phi_only<T, CANON>(P, Rp, zero, zj + d) - phi_only<T, CANON>(P, Rp, zero, zj - d)) * i2d;
        const T fm = density(P, Rm, zero, zj) * (phi_only<T, CANON>(P, Rm, zero, zj + d) - phi_only<T, CANON>(P, Rm, zero, zj - d)) * i2d;
        s0 += wj * f0;
        sp += wj * fp;
        sm += wj * fm;
    }
    s0 = warp_sum(s0) * dzq;
    sp = warp_sum(sp) * dzq;
    sm = warp_sum(sm) * dzq;
    if (lane != 0) return;
    const T nu = density(P, x, y, z);
    T vstream = 0, sR = 0, sz = 0;
    if (nu > T(0)) {
        const T sz2 = s0 / nu > T(0) ? s0 / nu : T(0);
        sz = M<T>::sqrt(sz2);
        sR = sz;   // anisotropy b = 1
        const T dP = (sp - sm) * i2d;
        const T dphidR = (phi_only<T, CANON>(P, R + d, zero, z) - phi_only<T, CANON>(P, R - d, zero, z)) * i2d;
        const T vphi2 = sz2 + (R / nu) * dP + R * dphidR;
        const T vs2 = vphi2 - sR * sR;
        vstream = vs2 > T(0) ? M<T>::sqrt(vs2) : T(0);
    }
    const T vR = normals[p] * sR;
    const T vz = normals[n + p] * sz;
    const T vphi = vstream + normals[2 * n + p] * sR;
    const T ph = M<T>::atan2(y, x);
    T sn, cs;
    if (sizeof(T) == 4) { float a, b; sincosf((float)ph, &a, &b); sn = a; cs = b; }
    else { double a, b; sincos((double)ph, &a, &b); sn = a; cs = b; }
    const T w[6] = {R * cs, R * sn, z, vR * cs + vphi * sn, vR * sn - vphi * cs, vz};
    if (w0_new)
        for (int c = 0; c < 6; ++c) w0_new[c * n + p] = w[c];
    // V_c and T_orb at the new position (dR = 1e-3)
    const T Rn = M<T>::sqrt(w[0] * w[0] + w[1] * w[1]);
    const T hR = T(1e-3);
    const T Rs = Rn > T(2) * hR ? Rn : T(2) * hR;
    const T dphi = (phi_only<T, CANON>(P, Rs + hR, zero, z) - phi_only<T, CANON>(P, Rs - hR, zero, z)) / (T(2) * hR);
    const T vc2 = Rs * dphi;
    const T Vc = vc2 > T(0) ? M<T>::sqrt(vc2) : T(0);
    T om2 = M<T>::abs(dphi) / Rs;
    om2 = om2 > T(1e-20) ? om2 : T(1e-20);
    const T Torb = T(2 * kPi) / M<T>::sqrt(om2);
    if (t_orb) t_orb[p] = Torb;
    if (vc) vc[p] = Vc;
    T vs = T(0.1) * Vc;
    vs = vs < T(1) ? T(1) : (vs > T(15) ? T(15) : vs);
    const T sc[6] = {T(0.1), T(0.1), T(0.1), vs, vs, vs};
    const int64_t n_orb = n * n_real;
    for (int r = 0; r < n_real; ++r) {
        const int64_t o = p * n_real + r;
        for (int c = 0; c < 6; ++c)
            w_out[c * n_orb + o] = w[c] + (unif[(c * n + p) * n_real + r] - T(0.5)) * sc[c];
        t_total[o] = Torb * n_periods;
        dt_init[o] = Torb / steps_pp;
    }
}

// One warp per cell (model.py:192-213).
template <typename T>
__global__ void density_target_kernel(PotT<T> P, const double *__restrict__ Rg, const double *__restrict__ zg,
                                      const double *__restrict__ pg, int64_t n_cells, double dR, double dz,
                                      double dphi, const double *__restrict__ smp, int n_s, T *out) {
    const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= n_cells) return;
    const T R0 = T(Rg[c]), z0 = T(zg[c]), p0 = T(pg[c]);
    const T tdR = T(dR), tdz = T(dz), tdp = T(dphi);
    T acc = 0;
    for (int j = lane; j < n_s; j += 32) {
        const T R = R0 + (T(smp[3 * j]) - T(0.5)) * tdR;
        const T zz = z0 + (T(smp[3 * j + 1]) - T(0.5)) * tdz;
        const T ph = p0 + (T(smp[3 * j + 2]) - T(0.5)) * tdp;
        T sn, cs;
        if (sizeof(T) == 4) { float a, b; sincosf((float)ph, &a, &b); sn = a; cs = b; }
        else { double a, b; sincos((double)ph, &a, &b); sn = a; cs = b; }
        acc += density(P, R * cs, R * sn, zz) * R;
    }
    acc = warp_sum(acc);
    if (lane == 0) out[c] = acc / T(n_s) * tdR * tdz * tdp;
}

static inline unsigned blocks_for(int64_t threads, int bs) { return (unsigned)((threads + bs - 1) / bs); }

}  // namespace smx

using namespace smx;

extern "C" {

int smx_potential_eval(const smx_potential *pot, int precision, const void *x, const void *y, const void *z,
                       int64_t n, void *phi, void *ax, void *ay, void *az, void *rho, void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (n < 0 || (n > 0 && (!x || !y || !z))) return set_error(SMX_ERR_ARGUMENT, "smx_potential_eval: bad points");
    if (n == 0) return SMX_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int bs = 128;
    if (precision == SMX_FP32) {
        potential_eval_kernel<float><<<blocks_for(n, bs), bs, 0, s>>>(make_pot<float>(*pot), (const float *)x,
            (const float *)y, (const float *)z, n, (float *)phi, (float *)ax, (float *)ay, (float *)az, (float *)rho);
        count_launch();
    } else if (precision == SMX_FP64) {
        potential_eval_kernel<double><<<blocks_for(n, bs), bs, 0, s>>>(make_pot<double>(*pot), (const double *)x,
            (const double *)y, (const double *)z, n, (double *)phi, (double *)ax, (double *)ay, (double *)az,
            (double *)rho);
        count_launch();
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

int smx_initial_conditions(const smx_potential *pot, int precision, const void *pos, const void *normals,
                           const void *uniforms, int64_t n, int n_real, double n_periods, double steps_per_period,
                           void *w_out, void *t_total, void *dt_init, void *w0_new, void *t_orb, void *vc,
                           void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (n < 0 || n_real < 1 || !(n_periods > 0) || !(steps_per_period > 0))
        return set_error(SMX_ERR_ARGUMENT, "smx_initial_conditions: bad sizes");
    if (n == 0) return SMX_OK;
    if (!pos || !normals || !uniforms || !w_out || !t_total || !dt_init)
        return set_error(SMX_ERR_ARGUMENT, "smx_initial_conditions: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const int bs = 128;
    const unsigned grid = blocks_for(n * 32, bs);
    const bool canon = canonical_types(*pot);
    if (precision == SMX_FP32) {
        auto kern = canon ? initial_conditions_kernel<float, true> : initial_conditions_kernel<float, false>;
        kern<<<grid, bs, 0, s>>>(make_pot<float>(*pot), (const float *)pos, (const float *)normals,
                                 (const float *)uniforms, n, n_real, (float)n_periods, (float)steps_per_period,
                                 (float *)w_out, (float *)t_total, (float *)dt_init, (float *)w0_new, (float *)t_orb,
                                 (float *)vc);
        count_launch();
    } else if (precision == SMX_FP64) {
        auto kern = canon ? initial_conditions_kernel<double, true> : initial_conditions_kernel<double, false>;
        kern<<<grid, bs, 0, s>>>(make_pot<double>(*pot), (const double *)pos, (const double *)normals,
                                 (const double *)uniforms, n, n_real, n_periods, steps_per_period, (double *)w_out,
                                 (double *)t_total, (double *)dt_init, (double *)w0_new, (double *)t_orb,
                                 (double *)vc);
        count_launch();
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

int smx_density_target(const smx_potential *pot, int precision, const double *R_grid, const double *z_grid,
                       const double *phi_grid, int64_t n_cells, double dR, double dz, double dphi,
                       const double *sample, int n_sample, void *out, void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (n_cells < 0 || n_sample < 1) return set_error(SMX_ERR_ARGUMENT, "smx_density_target: bad sizes");
    if (n_cells == 0) return SMX_OK;
    if (!R_grid || !z_grid || !phi_grid || !sample || !out)
        return set_error(SMX_ERR_ARGUMENT, "smx_density_target: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const int bs = 128;
    const unsigned grid = blocks_for(n_cells * 32, bs);
    if (precision == SMX_FP32) {
        density_target_kernel<float><<<grid, bs, 0, s>>>(make_pot<float>(*pot), R_grid, z_grid, phi_grid, n_cells,
                                                         dR, dz, dphi, sample, n_sample, (float *)out);
        count_launch();
    } else if (precision == SMX_FP64) {
        density_target_kernel<double><<<grid, bs, 0, s>>>(make_pot<double>(*pot), R_grid, z_grid, phi_grid,
                                                          n_cells, dR, dz, dphi, sample, n_sample, (double *)out);
        count_launch();
    } else {
        return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
    }
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

}  // extern "C"
