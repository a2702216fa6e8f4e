// Orbit integrator: adaptive Bogacki-Shampine 3(2) in the bar's rotating frame
// (integrates.py:8-238 for the stepper, the E_J record and the sampling rule).
//
// One thread owns one orbit at a time, with the state, the FSAL derivative and
// the step size in registers and the canonical forces evaluated inline.  Orbits
// are handed out by a device counter, so in the sampled mode (uneven step
// counts) a lane that finishes early takes the next orbit instead of idling,
// without leaving the loop the rest of its warp is in.
// Samples are written orbit-major, (7, n_orb, slots), so the projection kernel
// reads each orbit contiguously; consecutive writes of one thread land in the
// same sectors and merge in L2.
#include <mutex>
#include <vector>

#include "smx_internal.cuh"

namespace smx {

// The work counter and queue positions are int32: every lane takes one more
// position than it integrates, so n_orb + (resident threads) must stay below 2^31.
constexpr int64_t kMaxOrbits = ((int64_t)1 << 31) - ((int64_t)1 << 24);

template <typename T> struct IntegT {
    T atol, rtol, dt_min, dt_max, om;
    int mode, store_all, n_attempts, n_samples;
    long long max_attempts;
    const int32_t *order;   // queue position -> orbit (NULL: identity)
};

template <typename T, bool CANON>
__device__ __forceinline__ void rhs(const PotT<T> &P, T om, const T (&y)[6], T (&f)[6]) {
    T p, gx, gy, gz;
    potential<T, false, true, CANON>(P, y[0], y[1], y[2], p, gx, gy, gz);
    f[0] = y[3] + om * y[1];
    f[1] = y[4] - om * y[0];
    f[2] = y[5];
    f[3] = -gx + om * y[4];
    f[4] = -gy - om * y[3];
    f[5] = -gz;
}

template <typename T, bool CANON>
__device__ __forceinline__ T jacobi(const PotT<T> &P, T om, const T (&y)[6]) {
    const T ek = T(0.5) * (y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
    return ek + phi_only<T, CANON>(P, y[0], y[1], y[2]) - om * (y[0] * y[4] - y[1] * y[3]);
}

template <typename T>
__device__ __forceinline__ void put(T *samples, int64_t n_orb, int64_t slots, int64_t orb, int64_t slot,
                                    const T (&y)[6], T w) {
    T *base = samples + orb * slots + slot;
    const int64_t cs = n_orb * slots;
#pragma unroll
    for (int c = 0; c < 6; ++c) base[c * cs] = y[c];
    base[6 * cs] = w;
}

// k1 = f(y0) and E_J0 of every orbit, computed once before the main loop so
// that the loop never evaluates forces outside its attempt body.  k1 is parked
// in slot 0 of the orbit's sample store until the orbit is picked up (its
// first stored sample overwrites it later); E_J0 goes to its final place.
// Parameters of one parameter point of a batched call, in the working precision.
template <typename T> struct PointT {
    PotT<T> pot;
    T om;
};

template <typename T>
__device__ __forceinline__ PointT<T> make_point(const smx_point &p) {
    PointT<T> q;
    q.pot = make_pot<T>(p.pot);
    q.om = T(p.omega);
    return q;
}

template <typename T>
__global__ void __launch_bounds__(128) integrate_init_kernel(PotT<T> P0, T om0, const smx_point *__restrict__ points,
                                                            int64_t per_point, const T *__restrict__ w0,
                                                            int64_t n_orb, int64_t slots, T *samples, T *info) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n_orb) return;
    const PointT<T> pp = points ? make_point<T>(points[o / per_point]) : PointT<T>{P0, om0};
    const PotT<T> &P = pp.pot;
    const T om = pp.om;
    T y[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) y[c] = w0[c * n_orb + o];
    T phi, gx, gy, gz;
    potential<T, true, true>(P, y[0], y[1], y[2], phi, gx, gy, gz);
    const T f[6] = {y[3] + om * y[1], y[4] - om * y[0], y[5], -gx + om * y[4], -gy - om * y[3], -gz};
    const T ek = T(0.5) * (y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
    info[SMX_INFO_EJ0 * n_orb + o] = ek + phi - om * (y[0] * y[4] - y[1] * y[3]);
    T *base = samples + o * slots;
    const int64_t cs = n_orb * slots;
#pragma unroll
    for (int c = 0; c < 6; ++c) base[c * cs] = f[c];
}

// Main loop.  Every iteration is one BS23 attempt for every active lane: the
// three stage evaluations run through one inlined force evaluation inside a
// stage loop whose index is uniform across the warp, so the expensive part of
// the body is convergent even though lanes hold different orbits at different
// times.  A lane whose orbit ends (attempt cap, all samples emitted, stall or
// non-finite state) writes its record and loads the next orbit from the queue
// in the same iteration.
//
// BATCH: the orbits of n_points parameter points share one queue (orbit g belongs
// to point g / per_point); every block copies the points' potentials and frame
// rates into shared memory, and a lane reads those of its current orbit's point,
// so that one launch covers the whole batch and the uneven step counts of all its
// points even out across the SMs.
template <typename T, bool BATCH, bool CANON>
__global__ void __launch_bounds__(128) integrate_kernel(PotT<T> P0, IntegT<T> I, const smx_point *__restrict__ points,
                                                       int n_points, int64_t per_point, const T *__restrict__ w0,
                                                       const T *__restrict__ dt0, const T *__restrict__ t_end,
                                                       int64_t n_orb, int64_t slots, T *samples,
                                                       int32_t *n_stored, T *info, int32_t *status,
                                                       int32_t *queue) {
    extern __shared__ __align__(16) unsigned char pts_smem[];
    PointT<T> *spts = reinterpret_cast<PointT<T> *>(pts_smem);
    if (BATCH) {
        for (int i = threadIdx.x; i < n_points; i += blockDim.x) spts[i] = make_point<T>(points[i]);
        __syncthreads();
    }
    const T e1 = T(-5.0 / 72.0), e2 = T(1.0 / 12.0), e3 = T(1.0 / 9.0), e4 = T(-1.0 / 8.0);
    const T b1 = T(2.0 / 9.0), b2 = T(1.0 / 3.0), b3 = T(4.0 / 9.0);
    int pt = 0;   // parameter point of the current orbit (BATCH)
    const bool sampled = I.mode == SMX_MODE_SAMPLED;
    const int att_cap = sampled ? (int)(I.max_attempts < 0x7fffffffLL ? I.max_attempts : 0x7fffffffLL) : I.n_attempts;
    const int n_samp = I.n_samples;
    const int islots = (int)(slots < 0x7fffffffLL ? slots : 0x7fffffffLL);
    const int64_t cs = n_orb * slots;
    T y[6], k1[6], k2[6], k3[6], k4[6], yn[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) k2[c] = k3[c] = k4[c] = yn[c] = T(0);
    T dt = T(0), t = T(0), h = T(0), wsum = T(0);
    int att = 0, n_acc = 0, next = 0, flags = 0;
    // q: position in the work queue; orb: the orbit at that position (entries of
    // order outside [0, n_orb) are skipped, so a bad permutation cannot write
    // out of bounds)
    int q, orb = 0;
    auto take = [&]() {
        do {
            q = atomicAdd(queue, 1);
            orb = q < n_orb ? (I.order ? I.order[q] : q) : 0;
        } while (q < n_orb && (orb < 0 || orb >= n_orb));
    };
    take();

    auto load = [&](int o) {
        if (BATCH) pt = (int)(o / per_point);
        const T *base = samples + (int64_t)o * slots;
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            y[c] = w0[c * n_orb + o];
            k1[c] = base[c * cs];
        }
        dt = dt0[o];
        t = T(0);
        wsum = T(0);
        h = sampled ? t_end[o] / T(n_samp) : T(0);
        att = n_acc = next = flags = 0;
    };
    if (q < n_orb) load(orb);

    while (q < n_orb) {
        const PotT<T> &P = BATCH ? spts[pt].pot : P0;
        const T om = BATCH ? spts[pt].om : I.om;
        ++att;
        // stage inputs are formed as soon as their slopes exist, so the stage loop
        // body is one force evaluation plus a uniform branch on s
        T yt[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) yt[c] = y[c] + T(0.5) * dt * k1[c];
#pragma unroll 1
        for (int s = 0; s < 3; ++s) {
            T f[6];
            rhs<T, CANON>(P, om, yt, f);
            if (s == 0) {
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    k2[c] = f[c];
                    yt[c] = y[c] + T(0.75) * dt * f[c];
                }
            } else if (s == 1) {
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    k3[c] = f[c];
                    yn[c] = y[c] + dt * (b1 * k1[c] + b2 * k2[c] + b3 * f[c]);
                    yt[c] = yn[c];
                }
            } else {
#pragma unroll
                for (int c = 0; c < 6; ++c) k4[c] = f[c];
            }
        }
        T sq = T(0);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const T err = dt * (e1 * k1[c] + e2 * k2[c] + e3 * k3[c] + e4 * k4[c]);
            const T ay = M<T>::abs(y[c]), ayn = M<T>::abs(yn[c]);
            const T sc = I.atol + I.rtol * (ay > ayn ? ay : ayn);
            const T q = err * M<T>::rcp(sc);
            sq += q * q;
        }
        const T en = M<T>::sqrt(sq / T(6));
        if (!(en == en)) {
            flags |= 1;   // non-finite: the orbit is lost (it fails the E_J test downstream)
        } else {
            const bool accept = en <= T(1);
            if (accept) {
                ++n_acc;
                const T t1 = t + dt;
                if (sampled) {
                    const T idt = M<T>::rcp(dt);
                    // emit the sample times (j + 1/2) h inside (t, t1] by cubic Hermite
                    while (next < n_samp) {
                        const T tj = (T(next) + T(0.5)) * h;
                        if (tj > t1) break;
                        const T th = (tj - t) * idt;
                        const T th2 = th * th, th3 = th2 * th;
                        const T h00 = T(2) * th3 - T(3) * th2 + T(1);
                        const T h10 = (th3 - T(2) * th2 + th) * dt;
                        const T h01 = T(-2) * th3 + T(3) * th2;
                        const T h11 = (th3 - th2) * dt;
                        T ys[6];
#pragma unroll
                        for (int c = 0; c < 6; ++c) ys[c] = h00 * y[c] + h10 * k1[c] + h01 * yn[c] + h11 * k4[c];
                        if (next < islots) put(samples, n_orb, slots, orb, next, ys, h);
                        else flags |= 4;
                        wsum += h;
                        ++next;
                    }
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    y[c] = yn[c];
                    k1[c] = k4[c];
                }
                if (!sampled) {
                    const int slot = I.store_all ? att - 1 : next;
                    if (slot < islots) put(samples, n_orb, slots, orb, slot, y, dt);
                    else flags |= 4;
                    next = slot + 1;
                    wsum += dt;
                }
                t = t1;
            } else {
                if (!sampled && I.store_all) {
                    const int slot = att - 1;
                    if (slot < islots) put(samples, n_orb, slots, orb, slot, y, T(0));
                    else flags |= 4;
                    next = slot + 1;
                }
                if (dt <= I.dt_min) {
                    // Rejected at the smallest step: the next attempt repeats this one
                    // exactly (same y, k1 and dt = dt_min), so every later attempt is
                    // rejected too.  Stop here; a trajectory store gets the remaining
                    // attempts as the same zero-weight state.
                    flags |= 8;
                    if (!sampled && I.store_all) {
                        for (int slot = att; slot < att_cap && slot < islots; ++slot)
                            put(samples, n_orb, slots, orb, slot, y, T(0));
                        next = att_cap < islots ? att_cap : islots;
                    }
                }
            }
            T sf = T(0.9) * M<T>::rcbrt(en > T(1e-10) ? en : T(1e-10));
            sf = sf < T(0.2) ? T(0.2) : (sf > T(5) ? T(5) : sf);
            const T dn = dt * sf;
            dt = dn < I.dt_min ? I.dt_min : (dn > I.dt_max ? I.dt_max : dn);
        }
        const bool done = (flags & 9) || att >= att_cap || (sampled && next >= n_samp);
        if (done) {
            if (sampled && next < n_samp) flags |= 2;
            n_stored[orb] = next < islots ? next : islots;
            const T EJ = jacobi<T, CANON>(P, om, y);
            info[SMX_INFO_T * n_orb + orb] = t;
            info[SMX_INFO_EJ * n_orb + orb] = EJ;
            info[SMX_INFO_WSUM * n_orb + orb] = wsum;
            info[SMX_INFO_NACC * n_orb + orb] = T(n_acc);
            info[SMX_INFO_NATT * n_orb + orb] = T(att);
            status[orb] = flags;
            take();
            if (q < n_orb) load(orb);
        }
    }
}

template <typename T>
static IntegT<T> make_integ(const smx_integrator *cfg) {
    IntegT<T> I;
    I.atol = T(cfg->atol);
    I.rtol = T(cfg->rtol);
    I.dt_min = T(cfg->dt_min);
    I.dt_max = T(cfg->dt_max);
    I.om = T(cfg->omega);
    I.mode = cfg->mode;
    I.store_all = cfg->store_all;
    I.n_attempts = cfg->n_attempts;
    I.n_samples = cfg->n_samples;
    I.max_attempts = cfg->max_attempts;
    I.order = cfg->order;
    return I;
}

// points == NULL: one potential (pot, cfg->omega) for all orbits; otherwise the
// device array of n_points PointT<T> with per_point orbits each.
template <typename T>
static int launch(const smx_potential *pot, const smx_integrator *cfg, const smx_point *points, int n_points,
                  int64_t per_point, const void *w0, const void *dt_init, const void *t_total, int64_t n_orb,
                  int64_t slots, void *samples, int32_t *n_stored, void *info, int32_t *status, int32_t *queue,
                  int blocks_per_sm, cudaStream_t s) {
    const IntegT<T> I = make_integ<T>(cfg);
    const PotT<T> P0 = points ? PotT<T>() : make_pot<T>(*pot);
    const int64_t pp = per_point > 0 ? per_point : 1;
    SMX_TRY_CUDA(cudaMemsetAsync(queue, 0, sizeof(int32_t), s));
    integrate_init_kernel<T><<<(unsigned)((n_orb + 127) / 128), 128, 0, s>>>(P0, T(cfg->omega), points, pp,
                                                                         (const T *)w0, n_orb, slots,
                                                                         (T *)samples, (T *)info);
    count_launch();
    int dev = 0, sms = 0;
    SMX_TRY_CUDA(cudaGetDevice(&dev));
    SMX_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem = points ? (size_t)n_points * sizeof(PointT<T>) : 0;
    // the canonical model (T3 bar, V4 bulge) in every point: the compile-time fast path
    bool canon = true;
    if (points) {
        std::vector<smx_point> hp(n_points);
        SMX_TRY_CUDA(cudaMemcpyAsync(hp.data(), points, n_points * sizeof(smx_point), cudaMemcpyDeviceToHost, s));
        SMX_TRY_CUDA(cudaStreamSynchronize(s));
        for (const auto &q : hp) canon = canon && canonical_types(q.pot);
    } else {
        canon = canonical_types(*pot);
    }
    auto kern = points ? (canon ? integrate_kernel<T, true, true> : integrate_kernel<T, true, false>)
                       : (canon ? integrate_kernel<T, false, true> : integrate_kernel<T, false, false>);
    if (smem > 48 * 1024) SMX_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    SMX_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem));
    if (per_sm < 1) per_sm = 1;
    if (blocks_per_sm > 0 && blocks_per_sm < per_sm) per_sm = blocks_per_sm;
    // the same number of blocks on every SM: orbits come from the queue, so every
    // SM keeps working until the queue is empty (512 blocks for 65,536 orbits
    // would put 4 blocks on some SMs and 3 on others)
    int64_t bps = (n_orb + (int64_t)sms * 128 - 1) / ((int64_t)sms * 128);
    if (bps > per_sm) bps = per_sm;
    int64_t blocks = (int64_t)sms * bps;
    if (blocks > (n_orb + 127) / 128 * 2 && (n_orb + 127) / 128 < sms) blocks = (n_orb + 127) / 128;   // tiny calls
    kern<<<(unsigned)blocks, 128, smem, s>>>(P0, I, points, n_points, pp, (const T *)w0, (const T *)dt_init,
                                             (const T *)t_total, n_orb, slots, (T *)samples, n_stored, (T *)info,
                                             status, queue);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

static int validate_cfg(const smx_integrator *cfg, const void *t_total) {
    if (cfg->mode == SMX_MODE_REFERENCE) {
        if (cfg->n_attempts < 1) return set_error(SMX_ERR_ARGUMENT, "n_attempts must be >= 1");
    } else if (cfg->mode == SMX_MODE_SAMPLED) {
        if (cfg->n_samples < 1 || cfg->max_attempts < 1 || !t_total)
            return set_error(SMX_ERR_ARGUMENT, "sampled mode needs n_samples, max_attempts and t_total");
    } else {
        return set_error(SMX_ERR_ARGUMENT, "unknown integrator mode %d", cfg->mode);
    }
    if (!(cfg->atol > 0) || !(cfg->rtol >= 0) || !(cfg->dt_min > 0) || !(cfg->dt_max >= cfg->dt_min))
        return set_error(SMX_ERR_ARGUMENT, "bad tolerances or step bounds");
    return SMX_OK;
}

}  // namespace smx

using namespace smx;

extern "C" int smx_integrate(const smx_potential *pot, const smx_integrator *cfg, int precision, const void *w0,
                             const void *dt_init, const void *t_total, int64_t n_orb, int64_t slots, void *samples,
                             int32_t *n_stored, void *info, int32_t *status, int32_t *queue, void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (!cfg) return set_error(SMX_ERR_ARGUMENT, "smx_integrate: cfg is NULL");
    if (n_orb < 0 || slots < 1) return set_error(SMX_ERR_ARGUMENT, "smx_integrate: bad sizes");
    if (n_orb > kMaxOrbits)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_integrate: n_orb = %lld exceeds the 32-bit work counter's limit of %lld",
                         (long long)n_orb, (long long)kMaxOrbits);
    if (n_orb == 0) return SMX_OK;
    if (!w0 || !dt_init || !samples || !n_stored || !info || !status || !queue)
        return set_error(SMX_ERR_ARGUMENT, "smx_integrate: NULL buffer");
    if ((st = validate_cfg(cfg, t_total))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == SMX_FP32)
        return launch<float>(pot, cfg, nullptr, 0, 0, w0, dt_init, t_total, n_orb, slots, samples, n_stored, info,
                             status, queue, 0, s);
    if (precision == SMX_FP64)
        return launch<double>(pot, cfg, nullptr, 0, 0, w0, dt_init, t_total, n_orb, slots, samples, n_stored, info,
                              status, queue, 0, s);
    return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
}

extern "C" int smx_integrate_batch(const smx_point *points, int n_points, int64_t per_point,
                                   const smx_integrator *cfg, int precision, const void *w0, const void *dt_init,
                                   const void *t_total, int64_t slots, void *samples, int32_t *n_stored, void *info,
                                   int32_t *status, int32_t *queue, int blocks_per_sm, void *stream) {
    if (!cfg || !points) return set_error(SMX_ERR_ARGUMENT, "smx_integrate_batch: cfg or points is NULL");
    if (n_points < 1 || n_points > 1024 || per_point < 1 || slots < 1)
        return set_error(SMX_ERR_ARGUMENT, "smx_integrate_batch: bad sizes (1 <= n_points <= 1024)");
    const int64_t n_orb = (int64_t)n_points * per_point;
    if (n_orb > kMaxOrbits)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_integrate_batch: %lld orbits exceed the 32-bit work counter's limit",
                         (long long)n_orb);
    if (!w0 || !dt_init || !samples || !n_stored || !info || !status || !queue)
        return set_error(SMX_ERR_ARGUMENT, "smx_integrate_batch: NULL buffer");
    int st;
    if ((st = validate_cfg(cfg, t_total))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == SMX_FP32)
        return launch<float>(nullptr, cfg, points, n_points, per_point, w0, dt_init, t_total, n_orb, slots, samples,
                             n_stored, info, status, queue, blocks_per_sm, s);
    if (precision == SMX_FP64)
        return launch<double>(nullptr, cfg, points, n_points, per_point, w0, dt_init, t_total, n_orb, slots, samples,
                              n_stored, info, status, queue, blocks_per_sm, s);
    return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
}

// ---------------------------------------------------------------------------
// smx_integrate_noalloc: the same integration for callers that cannot allocate
// device memory themselves (a host runtime with a fixed memory pool, code that
// runs while allocation is forbidden, a binding without access to the CUDA
// allocator).  smx_integrate needs one int32 of caller scratch for its work
// queue; this variant keeps that counter in a static device array of the
// library instead, so the caller passes only inputs and outputs.
//
//   * Scratch: kNoAllocScratchInts int32 (256 bytes) per GPU, held by every
//     GPU that loads the library until the process exits; one counter is used.
//   * Limit: the counter is 32-bit, so n_orb is limited to kNoAllocMaxOrbits.
//   * Set-up: the first call on a device looks up the array's device address
//     with cudaGetSymbolAddress (the host-side name is only a stand-in); make
//     that first call before any stream capture.
//   * Every call zeroes the shared counter on its stream before the kernel;
//     calls that overlap on the GPU (different streams, or different host
//     threads on one device) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace smx {

constexpr int kNoAllocScratchInts = 64;
constexpr int64_t kNoAllocMaxOrbits = kMaxOrbits;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) int32_t g_noalloc_queue[kNoAllocScratchInts];

static int noalloc_queue_ptr(int32_t **out) {
    static std::mutex mu;
    static int32_t *ptrs[kNoAllocMaxDevices] = {nullptr};
    int dev = 0;
    SMX_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return set_error(SMX_ERR_UNSUPPORTED, "smx_integrate_noalloc: device %d beyond %d", dev, kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_queue);
        if (e != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress(g_noalloc_queue)");
        ptrs[dev] = (int32_t *)p;
    }
    *out = ptrs[dev];
    return SMX_OK;
}

}  // namespace smx

extern "C" int smx_integrate_noalloc(const smx_potential *pot, const smx_integrator *cfg, int precision,
                                     const void *w0, const void *dt_init, const void *t_total, int64_t n_orb,
                                     int64_t slots, void *samples, int32_t *n_stored, void *info, int32_t *status,
                                     void *stream) {
    int st = validate_potential(pot);
    if (st) return st;
    if (!cfg) return set_error(SMX_ERR_ARGUMENT, "smx_integrate_noalloc: cfg is NULL");
    if (n_orb < 0 || slots < 1) return set_error(SMX_ERR_ARGUMENT, "smx_integrate_noalloc: bad sizes");
    if (n_orb > kNoAllocMaxOrbits)
        return set_error(SMX_ERR_UNSUPPORTED,
                         "smx_integrate_noalloc: n_orb = %lld exceeds the static work counter's limit of %lld orbits",
                         (long long)n_orb, (long long)kNoAllocMaxOrbits);
    if (n_orb == 0) return SMX_OK;
    if (!w0 || !dt_init || !samples || !n_stored || !info || !status)
        return set_error(SMX_ERR_ARGUMENT, "smx_integrate_noalloc: NULL buffer");
    if ((st = validate_cfg(cfg, t_total))) return st;
    int32_t *queue = nullptr;
    st = noalloc_queue_ptr(&queue);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // launch<T> zeroes the counter on `s` before the kernel
    if (precision == SMX_FP32)
        return launch<float>(pot, cfg, nullptr, 0, 0, w0, dt_init, t_total, n_orb, slots, samples, n_stored, info,
                             status, queue, 0, s);
    if (precision == SMX_FP64)
        return launch<double>(pot, cfg, nullptr, 0, 0, w0, dt_init, t_total, n_orb, slots, samples, n_stored, info,
                              status, queue, 0, s);
    return set_error(SMX_ERR_ARGUMENT, "bad precision %d", precision);
}
