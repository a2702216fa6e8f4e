// FP64-accurate products on the bf16 tensor cores: the sliced GEMM kernel and
// the slicing kernels (method and number format in split_gemm.cuh).
//
// Kernel layout (one CTA per SM, stream-K over (output tile, k step) units; a k step
// is half a k tile, KS = 16, one MMA per slice pair):
//   warp 0      producer: one cp.async.bulk per slice and k step into a ring of as
//               many stages as fit in shared memory (the slices are stored in global
//               memory in the shared-memory tile layout, K-major core matrices, so a
//               half tile is one contiguous copy; no tensor map).  Only the slices
//               that take part in some pair s + t <= LMAX are loaded;
//   warp 1      owns the tensor memory and issues tcgen05.mma from one thread;
//   warps 2..9  epilogue: at the end of every exact chunk they read the level 2/3
//               accumulators (tcgen05.ld) into int32 running sums; at the end of
//               a tile's k range they add T and R to global memory with atomics.
// Tensor memory: level 2 at column 0, level 3 at 128, levels >= 4 at 256.
// Every wait is bounded by a clock deadline; on expiry the CTA records an error
// code and stops issuing work.  Before it leaves, the copy thread waits for its
// bulk copies still in flight and the MMA thread commits to a barrier and waits
// for its MMAs (bounded waits that ignore the abort), and only then is the tensor
// memory freed.
#include <cstdio>

#include "smx_internal.cuh"
#include "split_gemm.cuh"

namespace smx {
namespace split {

namespace dev {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor, no swizzle: lbo = byte stride between
// core matrices along K, sbo = along M/N; bit 46 = descriptor version.
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor kind::f16: D f32, A and B bf16, both K-major
__host__ __device__ constexpr uint32_t idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    return done != 0;
}

// wait for the phase of the given parity to complete, for at most ~2^31 cycles
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile int *abort_flag) {
    const uint32_t a = smem_u32(b);
    if (mbar_try(a, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try(a, parity)) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}

// wait for a phase that is certain to complete (copies or MMAs already issued),
// ignoring the abort flag, for at most ~2^30 cycles
__device__ __forceinline__ bool mbar_drain(uint64_t *b, uint32_t parity) {
    const uint32_t a = smem_u32(b);
    const long long t0 = clock64();
    while (!mbar_try(a, parity))
        if (clock64() - t0 > (1ll << 30)) return false;
    return true;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void ld8(uint32_t taddr, float *v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

}  // namespace dev

struct GemmParams {
    const __nv_bfloat16 *A, *B;
    int64_t a_slice, b_slice;            // elements between slices
    int64_t a_row_tiles, b_row_tiles, k_tiles;
    int64_t k_steps;                     // KS-wide k steps per output tile (2 k_tiles)
    int64_t M, N;                        // logical output size
    int64_t n_tiles_out;                 // output tiles along N
    int64_t units;                       // total (tile, k tile) units
    int lower_only;
    unsigned long long *T;
    float *R;
    int64_t ld;
    int *err;
    const int *skip;   // optional: the kernel returns at once when *skip != 0
};

// output tile index -> (row tile, column tile)
__device__ __forceinline__ void tile_coords(const GemmParams &p, int64_t tile, int64_t &mt, int64_t &nt) {
    if (!p.lower_only) {
        mt = tile % p.a_row_tiles;
        nt = tile / p.a_row_tiles;
    } else {   // lower-triangular tiles in row order: tile = mt (mt + 1) / 2 + nt
        int64_t r = (int64_t)((sqrt(8.0 * (double)tile + 1.0) - 1.0) * 0.5);
        while (r * (r + 1) / 2 > tile) --r;
        while ((r + 1) * (r + 2) / 2 <= tile) ++r;
        mt = r;
        nt = tile - r * (r + 1) / 2;
    }
}

// k per pipeline stage: KSUB MMAs of K = 16 (the first or second half of a KT tile for
// KSUB = 1, a whole tile for KSUB = 2)
template <int SA, int SB, int LMAX, int NT, int EXACT, int STAGES, int KSUB>
struct Cfg {
    static constexpr int KS = 16 * KSUB;
    // slices that take part in some pair s + t <= LMAX (the others are never loaded)
    static constexpr int UA = SA < LMAX - 1 ? SA : LMAX - 1;
    static constexpr int UB = SB < LMAX - 1 ? SB : LMAX - 1;
    static constexpr uint32_t A_STEP = MT * KS * 2;        // bytes of one slice's k step
    static constexpr uint32_t B_STEP = NT * KS * 2;
    static constexpr uint32_t STAGE = UA * A_STEP + UB * B_STEP;
    static constexpr uint32_t SMEM = STAGES * STAGE + 256;
    static constexpr int HALF = NT / 2;                     // columns per epilogue warp
    static constexpr int THREADS = 320;
    // tensor-memory columns per accumulator: EXACT exact levels + 1 rounded
    static constexpr int ACC_STRIDE = (NT + 31) / 32 * 32;
    // the exact levels' sums stay below 2^24 units over 1024 / (pairs per level) k
    static constexpr int MAXP = EXACT < (SA < SB ? SA : SB) ? EXACT : (SA < SB ? SA : SB);
    static constexpr int CHUNK_KS = (MAXP < 1 ? 1024 : 1024 / MAXP) / KS;
    static constexpr int OUT_KS = OUT_KT * KT / KS;
    static_assert(CHUNK_KS >= 1, "chunk");
    static_assert(KT % KS == 0, "stage k");
};

// ring depth: as many stages as fit in 227 KB next to the barriers, at most 8
template <int SA, int SB, int LMAX, int NT, int EXACT, int KSUB>
constexpr int stages_for() {
    constexpr uint32_t st = Cfg<SA, SB, LMAX, NT, EXACT, 1, KSUB>::STAGE;
    constexpr int n = (int)((232448u - 256u) / st);
    return n > 8 ? 8 : n;
}

template <int SA, int SB, int LMAX, int NT, int EXACT, int STAGES, int KSUB>
__global__ void __launch_bounds__(320, 1) gemm_kernel(const GemmParams p) {
    using C = Cfg<SA, SB, LMAX, NT, EXACT, STAGES, KSUB>;
    static_assert(NT % 16 == 0 && NT <= 128 && NT >= 16, "N tile");
    static_assert(C::HALF % 8 == 0, "epilogue columns in groups of 8");
    static_assert((EXACT + 1) * C::ACC_STRIDE <= 512, "tensor memory");
    static_assert(EXACT >= 1 && EXACT <= 5, "exact levels");
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *full = (uint64_t *)(smem + STAGES * C::STAGE);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;
    uint64_t *acc_empty = acc_full + 1;
    uint64_t *mma_done = acc_empty + 1;   // final commit of the MMA thread, waited on before dealloc
    uint32_t *tmem_holder = (uint32_t *)(mma_done + 1);
    volatile int *abort_flag = (volatile int *)(tmem_holder + 1);

    if (p.skip && *p.skip) return;   // uniform over the grid, before any barrier or allocation
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t u0 = p.units * blockIdx.x / gridDim.x, u1 = p.units * (blockIdx.x + 1) / gridDim.x;

    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; ++i) {
            dev::mbar_init(full + i, 1);
            dev::mbar_init(empty + i, 1);
        }
        dev::mbar_init(acc_full, 1);
        dev::mbar_init(acc_empty, 8);
        dev::mbar_init(mma_done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         dev::smem_u32(tmem_holder)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    dev::fence_before();
    __syncthreads();
    dev::fence_after();
    const uint32_t tmem = *tmem_holder;

    // The three roles walk the same units u0 .. u1 - 1 with running counters (k step
    // within the tile, ring stage and its phase) instead of 64-bit divisions per unit.
    // Flush schedule shared by the MMA issuer and the epilogue: after unit u, flush if
    // the chunk is full, the output flush distance is reached or the tile ends.
    if (warp == 0) {
        if (lane == 0) {
            int stage = 0;
            uint32_t par = 0;                        // parity of the ring round
            int64_t it = 0;
            int64_t tile = u0 / p.k_steps, ks = u0 % p.k_steps;
            int64_t mt, nt;
            tile_coords(p, tile, mt, nt);
            for (int64_t u = u0; u < u1; ++u, ++it) {
                // a stage is refilled once the MMAs of its previous round have completed
                if (it >= STAGES && !dev::mbar_wait(empty + stage, par ^ 1u, abort_flag)) {
                    atomicExch(p.err, 1);
                    *abort_flag = 1;
                    break;
                }
                // tiles are contiguous along k, so k step ks of row tile mt starts at
                // (mt k_steps + ks) MT KS elements of a slice
                unsigned char *sbase = smem + stage * C::STAGE;
                const __nv_bfloat16 *ga = p.A + (mt * p.k_steps + ks) * (MT * C::KS);
                const __nv_bfloat16 *gb = p.B + (nt * p.k_steps + ks) * (NT * C::KS);
                dev::mbar_expect_tx(full + stage, C::STAGE);
#pragma unroll
                for (int s = 0; s < C::UA; ++s)
                    dev::bulk_g2s(sbase + s * C::A_STEP, ga + s * p.a_slice, C::A_STEP, full + stage);
#pragma unroll
                for (int t = 0; t < C::UB; ++t)
                    dev::bulk_g2s(sbase + C::UA * C::A_STEP + t * C::B_STEP, gb + t * p.b_slice, C::B_STEP,
                                  full + stage);
                if (++stage == STAGES) {
                    stage = 0;
                    par ^= 1u;
                }
                if (++ks == p.k_steps) {
                    ks = 0;
                    tile_coords(p, ++tile, mt, nt);
                }
            }
            // no bulk copy may still be landing in shared memory when the CTA leaves:
            // wait for the last STAGES issued stages (each has exactly one phase
            // outstanding, since a stage is refilled only after it was consumed).
            // On the normal path these have completed already.
            for (int64_t j = (it > STAGES ? it - STAGES : 0); j < it; ++j)
                if (!dev::mbar_drain(full + (int)(j % STAGES), (uint32_t)((j / STAGES) & 1))) atomicExch(p.err, 5);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t ID = dev::idesc(MT, NT);
            constexpr uint32_t LBO_A = (MT / 8) * 128, LBO_B = (NT / 8) * 128, SBO = 128;
            // descriptors of stage 0's first slices; a stage or slice offset is added to
            // the address field (shared addresses stay below 2^18, so it cannot carry)
            const uint32_t s0 = dev::smem_u32(smem);
            const uint64_t a_desc0 = dev::desc(s0, LBO_A, SBO);
            const uint64_t b_desc0 = dev::desc(s0 + C::UA * C::A_STEP, LBO_B, SBO);
            int stage = 0;
            uint32_t par = 0;
            int64_t ks = u0 % p.k_steps;
            int since_chunk = 0, since_out = 0;
            uint32_t flushes = 0;
            uint32_t fresh = (1u << (EXACT + 1)) - 1;   // accumulators to overwrite on their next MMA
            bool pending = false;                       // a chunk flush whose read-out has not been confirmed
            // one unit's MMAs of the exact levels (EXACTS = true) or of the rounded one
            auto issue = [&](uint64_t ad0, uint64_t bd0, bool exacts) {
#pragma unroll
                for (int j = 0; j < KSUB; ++j) {
#pragma unroll
                    for (int s = 1; s <= C::UA; ++s) {
#pragma unroll
                        for (int t = 1; t <= C::UB; ++t) {
                            if (s + t <= LMAX && ((s + t - 2 < EXACT) == exacts)) {
                                const uint64_t ad = ad0 + (((s - 1) * C::A_STEP + j * 2 * LBO_A) >> 4);
                                const uint64_t bd = bd0 + (((t - 1) * C::B_STEP + j * 2 * LBO_B) >> 4);
                                const int acc = (s + t - 2) < EXACT ? (s + t - 2) : EXACT;
                                dev::mma(tmem + acc * C::ACC_STRIDE, ad, bd, ID, (fresh >> acc) & 1u ? 0u : 1u);
                                fresh &= ~(1u << acc);
                            }
                        }
                    }
                }
            };
            for (int64_t u = u0; u < u1; ++u) {
                if (!dev::mbar_wait(full + stage, par, abort_flag)) {
                    atomicExch(p.err, 2);
                    *abort_flag = 1;
                    break;
                }
                dev::fence_after();
                const uint64_t soff = (uint64_t)((stage * C::STAGE) >> 4);
                const uint64_t ad0 = a_desc0 + soff, bd0 = b_desc0 + soff;
                // the rounded level is not read at a chunk flush, so its MMAs go first
                // while the epilogue still reads the exact levels of the previous chunk
                issue(ad0, bd0, false);
                if (pending) {
                    if (!dev::mbar_wait(acc_empty, (flushes - 1) & 1, abort_flag)) {
                        atomicExch(p.err, 3);
                        *abort_flag = 1;
                        break;
                    }
                    dev::fence_after();
                    pending = false;
                }
                issue(ad0, bd0, true);
                dev::commit(empty + stage);
                if (++stage == STAGES) {
                    stage = 0;
                    par ^= 1u;
                }
                ++since_chunk;
                ++since_out;
                const bool tile_end = (ks == p.k_steps - 1) || (u + 1 == u1);
                if (++ks == p.k_steps) ks = 0;
                const bool out_flush = tile_end || since_out == C::OUT_KS;
                if (out_flush || since_chunk == C::CHUNK_KS) {
                    dev::commit(acc_full);
                    ++flushes;
                    fresh |= (1u << EXACT) - 1;
                    since_chunk = 0;
                    if (out_flush) {
                        // the rounded level is read too: wait before any further MMA
                        if (u + 1 < u1) {
                            if (!dev::mbar_wait(acc_empty, (flushes - 1) & 1, abort_flag)) {
                                atomicExch(p.err, 3);
                                *abort_flag = 1;
                                break;
                            }
                            dev::fence_after();
                        }
                        fresh |= 1u << EXACT;
                        since_out = 0;
                    } else {
                        pending = true;
                    }
                }
            }
            // every MMA this thread issued must be complete before the tensor memory
            // is released, also when the loop above gave up early
            dev::commit(mma_done);
            if (!dev::mbar_drain(mma_done, 0)) atomicExch(p.err, 6);
        }
    } else {
        // epilogue: warp w reads lanes 32 (w % 4) .. + 31 (its row quarter), column half h.
        // The exact levels of a chunk are combined into one int64 per column in units
        // of 2^-8(EXACT-1): level 2 + e holds multiples of 2^-8e below 2^24 units.
        const int q = warp & 3, h = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * C::HALF);
        long long sum[C::HALF];
#pragma unroll
        for (int c = 0; c < C::HALF; ++c) sum[c] = 0;
        int since_chunk = 0, since_out = 0;
        uint32_t flushes = 0;
        int64_t ks = u0 % p.k_steps;
        for (int64_t u = u0; u < u1; ++u) {
            ++since_chunk;
            ++since_out;
            const bool tile_end = (ks == p.k_steps - 1) || (u + 1 == u1);
            if (++ks == p.k_steps) ks = 0;
            const bool out_flush = tile_end || since_out == C::OUT_KS;
            if (!(out_flush || since_chunk == C::CHUNK_KS)) continue;
            // every lane waits, and the warp goes on only if all of them saw the phase
            // complete, so that the .sync.aligned tensor-memory loads below run with the
            // full warp or not at all
            const bool seen = dev::mbar_wait(acc_full, flushes & 1, abort_flag);
            if (!__all_sync(0xffffffffu, seen)) {
                if (lane == 0) {
                    atomicExch(p.err, 4);
                    *abort_flag = 1;
                }
                break;
            }
            ++flushes;
            dev::fence_after();
            int64_t mt = 0, nt = 0;
            if (out_flush) tile_coords(p, u / p.k_steps, mt, nt);
            const int64_t gi = mt * MT + row;
#pragma unroll
            for (int c0 = 0; c0 < C::HALF; c0 += 8) {
                float v[EXACT][8], vr[8];
#pragma unroll
                for (int e = 0; e < EXACT; ++e) dev::ld8(lane_addr + e * C::ACC_STRIDE + c0, v[e]);
                if (out_flush) dev::ld8(lane_addr + EXACT * C::ACC_STRIDE + c0, vr);
                dev::ld_wait();
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    long long add = 0;
#pragma unroll
                    for (int e = 0; e < EXACT; ++e)   // level 2 + e in units of 2^-8e: scale by 2^8e (exact)
                        add += (long long)__float2int_rn(v[e][j] * __int_as_float((127 + 8 * e) << 23))
                               << (8 * (EXACT - 1 - e));
                    sum[c0 + j] += add;
                }
                if (out_flush) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int64_t gj = nt * NT + h * C::HALF + c0 + j;
                        if (gi < p.M && gj < p.N) {
                            atomicAdd(p.T + gi + p.ld * gj, (unsigned long long)sum[c0 + j]);
                            atomicAdd(p.R + gi + p.ld * gj, vr[j]);
                        }
                        sum[c0 + j] = 0;
                    }
                }
            }
            dev::fence_before();
            __syncwarp();
            if (lane == 0) dev::mbar_arrive(acc_empty);
            since_chunk = 0;
            if (out_flush) since_out = 0;
        }
    }
    dev::fence_before();
    __syncthreads();
    if (warp == 1) {
        dev::fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

// ------------------------------------------------------------------ slicing

// max |x| per row, as the bits of a non-negative double (ordered like the values)
template <typename T>
__global__ void rowmax_kernel(const T *__restrict__ src, int64_t sr, int64_t sc, int64_t rows, int64_t k,
                              unsigned long long *rowmax, int rows_fast, int skip_diag, const int *skip) {
    if (skip && *skip) return;
    if (rows_fast) {   // consecutive threads on consecutive rows; blocks along k
        const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        if (r >= rows) return;
        const int64_t kc = (k + gridDim.y - 1) / gridDim.y;
        const int64_t k0 = blockIdx.y * kc, k1 = k0 + kc < k ? k0 + kc : k;
        double m = 0;
        for (int64_t c = k0; c < k1; ++c)
            if (!(skip_diag && c == r)) m = fmax(m, fabs((double)src[r * sr + c * sc]));
        atomicMax(rowmax + r, (unsigned long long)__double_as_longlong(m));
    } else {           // one warp per row, lanes along k
        const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        const int lane = threadIdx.x & 31;
        if (r >= rows) return;
        double m = 0;
        for (int64_t c = lane; c < k; c += 32)
            if (!(skip_diag && c == r)) m = fmax(m, fabs((double)src[r * sr + c * sc]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) atomicMax(rowmax + r, (unsigned long long)__double_as_longlong(m));
    }
}

// e with max < 2^e (0 for an all-zero row)
__device__ __forceinline__ int scale_exponent(double mx) {
    if (!(mx > 0)) return 0;
    int e;
    frexp(mx, &e);   // mx = f 2^e, f in [0.5, 1)
    return e;
}

__global__ void expo_kernel(const unsigned long long *rowmax, int32_t *expo, int64_t rows, int64_t rows_padded,
                            const int *skip) {
    if (skip && *skip) return;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows_padded; r += (int64_t)gridDim.x * blockDim.x)
        expo[r] = r < rows ? scale_exponent(__longlong_as_double((long long)rowmax[r])) : 0;
}

// one CTA per (row tile, k tile): builds the S slice tiles in shared memory and
// writes each as contiguous 16-byte vectors
template <typename T, int S>
__global__ void slice_rows_kernel(const T *__restrict__ src, int64_t sr, int64_t sc, int64_t rows, int64_t k,
                                  const int32_t *__restrict__ expo, __nv_bfloat16 *slices, int tile_rows,
                                  int64_t k_tiles, int64_t slice_elems, int k_fast, int skip_diag, const int *skip) {
    if (skip && *skip) return;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    __nv_bfloat16 *tile = (__nv_bfloat16 *)sm_raw;   // S x tile_rows x KT
    const int64_t kt = blockIdx.x, rt = blockIdx.y;
    const int n = tile_rows * KT;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        int r, c;
        if (k_fast) {
            c = idx % KT;
            r = idx / KT;
        } else {
            r = idx % tile_rows;
            c = idx / tile_rows;
        }
        const int64_t gr = rt * tile_rows + r, gc = kt * KT + c;
        double x = 0;
        int e = 0;
        if (gr < rows && gc < k && !(skip_diag && gr == gc)) {
            x = (double)src[gr * sr + gc * sc];
            e = expo[gr];
        }
        __nv_bfloat16 v[S];
        make_slices<S>(x, e, v);
        const int64_t off = tile_offset(r, c, tile_rows);
#pragma unroll
        for (int s = 0; s < S; ++s) tile[s * n + off] = v[s];
    }
    __syncthreads();
    const int vec = n / 8;   // 16-byte vectors per slice tile
    for (int idx = threadIdx.x; idx < S * vec; idx += blockDim.x) {
        const int s = idx / vec, v = idx % vec;
        const uint4 w = ((const uint4 *)(tile + s * n))[v];
        ((uint4 *)(slices + s * slice_elems + (rt * k_tiles + kt) * n))[v] = w;
    }
}

// ------------------------------------------------------------------ host side

// Stages of a whole KT tile (two MMAs of K = 16 per slice pair).  Half-tile stages fit
// twice as many stages in shared memory, but ran the config-1 NNLS 10 % slower
// (200 ms against 182 ms per solve on one GB300).
constexpr int kStageSub = 2;

template <int SA, int SB, int LMAX, int NT, int EXACT>
static int launch_gemm(const Operand &A, const Operand &B, const Acc &acc, bool lower_only, int *err, cudaStream_t s,
                       const int *skip) {
    constexpr int KSUB = kStageSub;
    constexpr int STAGES = stages_for<SA, SB, LMAX, NT, EXACT, KSUB>();
    using C = Cfg<SA, SB, LMAX, NT, EXACT, STAGES, KSUB>;
    static_assert(STAGES >= 2 && C::SMEM <= 232448, "shared memory");
    SMX_TRY_CUDA(cudaFuncSetAttribute(gemm_kernel<SA, SB, LMAX, NT, EXACT, STAGES, KSUB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM));
    int dev = 0, sms = 0;
    SMX_TRY_CUDA(cudaGetDevice(&dev));
    SMX_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GemmParams p;
    p.A = A.slices;
    p.B = B.slices;
    p.a_slice = A.slice_elems();
    p.b_slice = B.slice_elems();
    p.a_row_tiles = A.row_tiles;
    p.b_row_tiles = B.row_tiles;
    p.k_tiles = A.k_tiles;
    p.k_steps = A.k_tiles * (KT / C::KS);
    p.M = A.rows;
    p.N = B.rows;
    p.n_tiles_out = B.row_tiles;
    p.lower_only = lower_only ? 1 : 0;
    const int64_t tiles = lower_only ? A.row_tiles * (A.row_tiles + 1) / 2 : A.row_tiles * B.row_tiles;
    p.units = tiles * p.k_steps;
    p.T = acc.T;
    p.R = acc.R;
    p.ld = acc.ld;
    p.err = err;
    p.skip = skip;
    int64_t grid = sms;
    if (grid > p.units) grid = p.units;
    gemm_kernel<SA, SB, LMAX, NT, EXACT, STAGES, KSUB><<<(unsigned)grid, C::THREADS, C::SMEM, s>>>(p);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

int exact_levels(const Operand &A, const Operand &B) {
    if (A.S == 7 && B.S == 7) return 4;
    if (A.S == 2 && B.S == 2) return 2;
    return B.tile_rows == 64 ? 5 : 3;
}

// Kernel configurations: every slice pair is formed (LMAX = SA + SB).  Column
// tiles of 112 or 128 leave room for three exact levels (four accumulators of
// 128 tensor-memory columns); 64-wide tiles for five (six accumulators), for
// operands whose rows are dominated by one element (an inverse's diagonal);
// 7 x 7 slices use pairs up to s + t = 8, four exact levels and 96-wide tiles.
int gemm(const Operand &A, const Operand &B, const Acc &acc, bool lower_only, int *err, cudaStream_t s, int lmax,
         const int *skip) {
    if (!A.slices || !A.expo || !B.slices || !B.expo || !acc.T || !acc.R || !err)
        return set_error(SMX_ERR_ARGUMENT, "split gemm: operand or accumulator without storage");
    if (acc.ld < A.rows) return set_error(SMX_ERR_ARGUMENT, "split gemm: accumulator leading dimension too small");
    if (A.k_tiles != B.k_tiles || A.tile_rows != MT)
        return set_error(SMX_ERR_ARGUMENT, "split gemm: operand shapes do not match");
    if (lower_only && B.tile_rows != MT) return set_error(SMX_ERR_ARGUMENT, "split gemm: lower_only needs square tiles");
    const int key = A.S * 10 + B.S;
    if (B.tile_rows == 112 && key == 45 && lmax == 7)
        return launch_gemm<4, 5, 7, 112, 3>(A, B, acc, lower_only, err, s, skip);
    if (B.tile_rows == 112 && key == 45 && lmax == 6)
        return launch_gemm<4, 5, 6, 112, 3>(A, B, acc, lower_only, err, s, skip);
    if (B.tile_rows == 112 && key == 45 && lmax == 5)
        return launch_gemm<4, 5, 5, 112, 3>(A, B, acc, lower_only, err, s, skip);
    if (B.tile_rows == 128 && key == 54 && lmax == 6)
        return launch_gemm<5, 4, 6, 128, 3>(A, B, acc, lower_only, err, s, skip);
    if (B.tile_rows == 128 && key == 44 && lmax == 5)
        return launch_gemm<4, 4, 5, 128, 3>(A, B, acc, lower_only, err, s, skip);
    if (B.tile_rows == 128 && key == 55 && lmax == 6)
        return launch_gemm<5, 5, 6, 128, 3>(A, B, acc, lower_only, err, s, skip);
    if (B.tile_rows == 96 && key == 77 && lmax == 7)
        return launch_gemm<7, 7, 7, 96, 4>(A, B, acc, lower_only, err, s, skip);
    if (lmax != 0) return set_error(SMX_ERR_UNSUPPORTED, "split gemm: no kernel with pairs up to s + t = %d", lmax);
    if (B.tile_rows == 112) {
        switch (key) {
            case 22: return launch_gemm<2, 2, 4, 112, 2>(A, B, acc, lower_only, err, s, skip);
            case 33: return launch_gemm<3, 3, 6, 112, 3>(A, B, acc, lower_only, err, s, skip);
            case 44: return launch_gemm<4, 4, 8, 112, 3>(A, B, acc, lower_only, err, s, skip);
            case 45: return launch_gemm<4, 5, 9, 112, 3>(A, B, acc, lower_only, err, s, skip);
            case 54: return launch_gemm<5, 4, 9, 112, 3>(A, B, acc, lower_only, err, s, skip);
            case 55: return launch_gemm<5, 5, 10, 112, 3>(A, B, acc, lower_only, err, s, skip);
            default: break;
        }
    } else if (B.tile_rows == 128) {
        switch (key) {
            case 44: return launch_gemm<4, 4, 8, 128, 3>(A, B, acc, lower_only, err, s, skip);
            case 54: return launch_gemm<5, 4, 9, 128, 3>(A, B, acc, lower_only, err, s, skip);
            case 55: return launch_gemm<5, 5, 10, 128, 3>(A, B, acc, lower_only, err, s, skip);
            default: break;
        }
    } else if (B.tile_rows == 96) {
        if (key == 77) return launch_gemm<7, 7, 8, 96, 4>(A, B, acc, lower_only, err, s, skip);
    } else if (B.tile_rows == 64) {
        if (key == 55) return launch_gemm<5, 5, 10, 64, 5>(A, B, acc, lower_only, err, s, skip);
    }
    return set_error(SMX_ERR_UNSUPPORTED, "split gemm: no kernel for %d x %d slices with %d-row column tiles", A.S, B.S,
                     B.tile_rows);
}

static inline unsigned grid_for(int64_t count, int bs) {
    int64_t g = (count + bs - 1) / bs;
    if (g > 152 * 64) g = 152 * 64;
    return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
int slice_rows(const T *src, int64_t sr, int64_t sc, const Operand &op, unsigned long long *rowmax, cudaStream_t s,
               bool skip_diag, const int *skip) {
    if (!src || !op.slices || !op.expo || !rowmax)
        return set_error(SMX_ERR_ARGUMENT, "slice_rows: operand without storage");
    const int64_t rows_padded = op.row_tiles * op.tile_rows;
    SMX_TRY_CUDA(cudaMemsetAsync(rowmax, 0, sizeof(unsigned long long) * op.rows, s));
    // rows contiguous in memory (sr == 1): threads along rows; else a warp per row along k
    const bool rows_fast = sr == 1;
    if (rows_fast) {
        dim3 g((unsigned)((op.rows + 255) / 256), (unsigned)(op.k < 64 ? op.k : 64));
        rowmax_kernel<T><<<g, 256, 0, s>>>(src, sr, sc, op.rows, op.k, rowmax, 1, skip_diag ? 1 : 0, skip);
    } else {
        rowmax_kernel<T><<<grid_for(op.rows * 32, 256), 256, 0, s>>>(src, sr, sc, op.rows, op.k, rowmax, 0,
                                                                   skip_diag ? 1 : 0, skip);
    }
    count_launch();
    expo_kernel<<<grid_for(rows_padded, 256), 256, 0, s>>>(rowmax, op.expo, op.rows, rows_padded, skip);
    count_launch();
    dim3 g((unsigned)op.k_tiles, (unsigned)op.row_tiles);
    const size_t sm = (size_t)op.S * op.tile_rows * KT * sizeof(__nv_bfloat16);
    const int k_fast = sc == 1 ? 1 : 0;
    switch (op.S) {
#define SMX_SLICE_CASE(NS)                                                                                       \
    case NS:                                                                                                    \
        SMX_TRY_CUDA(cudaFuncSetAttribute(slice_rows_kernel<T, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                          (int)sm));                                                             \
        slice_rows_kernel<T, NS><<<g, 256, sm, s>>>(src, sr, sc, op.rows, op.k, op.expo, op.slices, op.tile_rows,  \
                                                    op.k_tiles, op.slice_elems(), k_fast, skip_diag ? 1 : 0, skip); \
        break;
        SMX_SLICE_CASE(4)
        SMX_SLICE_CASE(5)
        SMX_SLICE_CASE(7)
#undef SMX_SLICE_CASE
        default: return set_error(SMX_ERR_UNSUPPORTED, "slice_rows: %d slices", op.S);
    }
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    return SMX_OK;
}

template int slice_rows<float>(const float *, int64_t, int64_t, const Operand &, unsigned long long *, cudaStream_t,
                               bool, const int *);
template int slice_rows<double>(const double *, int64_t, int64_t, const Operand &, unsigned long long *, cudaStream_t,
                                bool, const int *);

}  // namespace split
}  // namespace smx

// ------------------------------------------------------------ C ABI (products)

namespace smx {
namespace split {

__global__ void combine_kernel(const unsigned long long *T, const float *R, const int32_t *eA, const int32_t *eB,
                               double *C, int64_t M, int64_t N, int t_shift) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < M * N; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k % M, j = k / M;
        const double v = ldexp((double)(long long)T[k], -t_shift) + (double)R[k];
        C[k] = ldexp(v, eA[i] + eB[j] - 14);
    }
}

struct ProductLayout {
    Operand A, B;
    size_t a_sl, a_e, b_sl, b_e, T, R, rowmax, err, total;
};

static int product_layout(int64_t M, int64_t N, int64_t K, int sa, int sb, ProductLayout *L) {
    const bool ab45 = (sa == 4 || sa == 5) && (sb == 4 || sb == 5), square = (sa == 4 && sb == 4) || (sa == 5 && sb == 5);
    int bt;
    if (sa == 5 && sb == 5 && N <= 128) bt = 64;
    else if (N <= 112 && ab45) bt = 112;
    else if (square) bt = 128;
    else if (sa == 7 && sb == 7) bt = 96;
    else return set_error(SMX_ERR_UNSUPPORTED, "smx_split_gemm: slices %d x %d with N = %lld", sa, sb, (long long)N);
    L->A = make_operand(M, K, MT, sa);
    L->B = make_operand(N, K, bt, sb);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    L->a_sl = take(L->A.slice_bytes());
    L->a_e = take(L->A.row_tiles * MT * sizeof(int32_t));
    L->b_sl = take(L->B.slice_bytes());
    L->b_e = take(L->B.row_tiles * bt * sizeof(int32_t));
    L->T = take(M * N * sizeof(unsigned long long));
    L->R = take(M * N * sizeof(float));
    L->rowmax = take((M > N ? M : N) * sizeof(unsigned long long));
    L->err = take(sizeof(int) * 4);
    L->total = off;
    return SMX_OK;
}

}  // namespace split
}  // namespace smx

using namespace smx;

extern "C" int smx_split_gemm_workspace_size(int64_t M, int64_t N, int64_t K, int a_slices, int b_slices,
                                             size_t *bytes) {
    if (!bytes || M < 1 || N < 1 || K < 1) return set_error(SMX_ERR_ARGUMENT, "smx_split_gemm_workspace_size: bad argument");
    split::ProductLayout L;
    int st = split::product_layout(M, N, K, a_slices, b_slices, &L);
    if (st) return st;
    *bytes = L.total;
    return SMX_OK;
}

extern "C" int smx_split_gemm(int64_t M, int64_t N, int64_t K, int a_slices, int b_slices, int lower, const double *A,
                              const double *B, double *C, void *workspace, size_t workspace_bytes, void *stream) {
    if (M < 1 || N < 1 || K < 1 || !A || !B || !C || !workspace)
        return set_error(SMX_ERR_ARGUMENT, "smx_split_gemm: bad argument");
    if (M * N > ((int64_t)1 << 31) || M * K > ((int64_t)1 << 33) || N * K > ((int64_t)1 << 33))
        return set_error(SMX_ERR_UNSUPPORTED, "smx_split_gemm: problem too large");
    split::ProductLayout L;
    int st = split::product_layout(M, N, K, a_slices, b_slices, &L);
    if (st) return st;
    if (lower && (M != N || L.B.tile_rows != split::MT))
        return set_error(SMX_ERR_ARGUMENT, "smx_split_gemm: lower needs M == N and 128-row tiles");
    if (workspace_bytes < L.total)
        return set_error(SMX_ERR_WORKSPACE, "smx_split_gemm: workspace %zu < %zu bytes", workspace_bytes, L.total);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *ws = (unsigned char *)workspace;
    split::Operand a = L.A, b = L.B;
    a.slices = (__nv_bfloat16 *)(ws + L.a_sl);
    a.expo = (int32_t *)(ws + L.a_e);
    b.slices = (__nv_bfloat16 *)(ws + L.b_sl);
    b.expo = (int32_t *)(ws + L.b_e);
    unsigned long long *T = (unsigned long long *)(ws + L.T);
    float *R = (float *)(ws + L.R);
    int *err = (int *)(ws + L.err);
    SMX_TRY_CUDA(cudaMemsetAsync(T, 0, M * N * sizeof(unsigned long long), s));
    SMX_TRY_CUDA(cudaMemsetAsync(R, 0, M * N * sizeof(float), s));
    SMX_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    // A rows i over k: A[i + M k];  B^T rows j over k: B[k + K j]
    if ((st = split::slice_rows<double>(A, 1, M, a, (unsigned long long *)(ws + L.rowmax), s))) return st;
    if ((st = split::slice_rows<double>(B, K, 1, b, (unsigned long long *)(ws + L.rowmax), s))) return st;
    split::Acc acc{T, R, M};
    if ((st = split::gemm(a, b, acc, lower != 0, err, s))) return st;
    const int shift = 8 * (split::exact_levels(a, b) - 1);
    split::combine_kernel<<<split::grid_for(M * N, 256), 256, 0, s>>>(T, R, a.expo, b.expo, C, M, N, shift);
    count_launch();
    SMX_TRY_CUDA(cudaGetLastError());
    int herr = 0;
    SMX_TRY_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SMX_TRY_CUDA(cudaStreamSynchronize(s));
    if (herr) return set_error(SMX_ERR_CUDA, "smx_split_gemm: product kernel gave up waiting (code %d)", herr);
    return SMX_OK;
}
