// FP64-accurate matrix products on the bf16 tensor cores (Ozaki splitting).
//
// Method: Ozaki, Ogita, Oishi and Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012); on tensor cores with FP32
// accumulation as in Mukunoki, Ozaki, Ogita and Imamura, "DGEMM using Tensor
// Cores, and Its Accurate and Reproducible Versions", ISC 2020.
//
// Every row x of an operand is written with one power-of-two scale 2^e
// (max |x| < 2^e) as a sum of S slices,
//     x = 2^(e-7) * sum_s a'_s,    a'_s = a_s 2^(-8(s-1)),  a_s integer in [-128, 128],
// so every slice value is exact in bf16 and every slice product is exact in FP32.
// The product of two such operands is the sum over slice pairs (s, t) of
// A'_s B'_t^T, weighted 2^(-8(s+t-2)) relative to the leading pair.  Pairs with
// s + t <= LMAX are formed on the tensor cores (tcgen05.mma kind::f16, bf16
// inputs, FP32 accumulation in tensor memory):
//   levels 2 .. EXACT+1 each have an accumulator; level 2 + e holds multiples of
//   2^-8e, and over a chunk of 1024 / (pairs of the level) k its sum stays below
//   2^24 of those units, so the FP32 accumulation is exact.  At the end of every
//   chunk the exact levels are combined into one int64 running sum per output
//   (units 2^-8(EXACT-1)), which is exact as well;
//   the remaining levels share one FP32 accumulator.
// Rows with one dominant element (the diagonal of an inverse) carry most of a
// product in the lower levels, and the tensor cores' FP32 accumulation there
// leaves a systematic error, so by default every slice pair is formed
// (LMAX = SA + SB) with three exact levels (column tiles of 112 or 128) or five
// (64-wide tiles); 7 x 7 products use four exact levels.  Callers whose operands
// have no dominant element drop the pairs above a level (lmax below).
// The result for output (i, j) is returned as the exact int64 T and a float R,
// both accumulated with atomics over the k ranges of all CTAs, and the consumer
// forms   C_ij = 2^(eA_i + eB_j - 14) (T_ij 2^-8(EXACT-1) + R_ij)   in double.
// The remaining error is the slicing of the inputs: 2^-31 (4 slices) or 2^-39
// (5 slices) of each row's and column's largest magnitude.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace smx {
namespace split {

constexpr int KT = 32;          // k per stored tile (the product kernel stages half a tile at a time)
constexpr int MT = 128;         // rows of an A tile (MMA M)
constexpr int OUT_KT = 256;     // k tiles between output flushes at most: 8192 k (int64 running sums)

// bf16 element offset of (row r, column k) inside a rows x KT tile stored as
// 8 x 8 core matrices, core matrix (rg, kg) at ((kg * rows/8) + rg) * 64 elements
__host__ __device__ inline int64_t tile_offset(int r, int k, int rows) {
    return ((int64_t)((k >> 3) * (rows >> 3) + (r >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

// round(x 2^k) as an integer, from the bits of x (round half to even; |result|
// must stay below 2^62).  Integer arithmetic only: GB300's FP64 rate is low.
__device__ __forceinline__ long long to_fixed(double x, int k) {
    const long long b = __double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7FF);
    if (E == 0) return 0;                               // zero (and subnormals, < 2^-1022)
    const long long m = (b & ((1LL << 52) - 1)) | (1LL << 52);
    const int sh = E - 1075 + k;                        // x 2^k = m 2^sh
    long long v;
    if (sh >= 0) {
        v = m << sh;
    } else if (sh < -54) {
        v = 0;
    } else {
        const int r = -sh;
        const long long q = m >> r, rem = m & ((1LL << r) - 1), half = 1LL << (r - 1);
        v = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    }
    return b < 0 ? -v : v;
}
__device__ __forceinline__ long long to_fixed(float x, int k) { return to_fixed((double)x, k); }

// S slices of a value already scaled to a signed integer v, |v| <= 2^(7 + 8(S-1)):
// balanced base-256 digits a_s in [-128, 128], v = sum a_s 256^(S-1-s), stored as
// bf16 a_s 2^-8s (exact).
template <int S>
__device__ __forceinline__ void digits(long long v, __nv_bfloat16 *out) {
#pragma unroll
    for (int s = S - 1; s > 0; --s) {
        int d = (int)(v & 0xFF);
        v >>= 8;                                        // arithmetic shift: floor division
        if (d > 128) {
            d -= 256;
            v += 1;
        }
        out[s] = __float2bfloat16_rn(__int_as_float((127 - 8 * s) << 23) * (float)d);
    }
    out[0] = __float2bfloat16_rn((float)v);
}

// slices of x with scale exponent e (|x| < 2^e): x 2^(7 + 8(S-1) - e) rounded
template <int S, typename T>
__device__ __forceinline__ void make_slices(T x, int e, __nv_bfloat16 *out) {
    digits<S>(to_fixed(x, 7 + 8 * (S - 1) - e), out);
}

// Sliced operand: rows x k values as S bf16 slices in K-major tiles of
// tile_rows x KT, tiles ordered [slice][row tile][k tile]; expo[row] = e.
struct Operand {
    __nv_bfloat16 *slices = nullptr;
    int32_t *expo = nullptr;
    int64_t rows = 0, k = 0;       // logical
    int tile_rows = MT;
    int S = 0;
    int64_t row_tiles = 0, k_tiles = 0;
    int64_t slice_elems() const { return row_tiles * k_tiles * (int64_t)tile_rows * KT; }
    size_t slice_bytes() const { return (size_t)S * slice_elems() * sizeof(__nv_bfloat16); }
};

inline Operand make_operand(int64_t rows, int64_t k, int tile_rows, int S) {
    Operand o;
    o.rows = rows;
    o.k = k;
    o.tile_rows = tile_rows;
    o.S = S;
    o.row_tiles = (rows + tile_rows - 1) / tile_rows;
    o.k_tiles = (k + KT - 1) / KT;
    return o;
}

// Result accumulators of a product: T (int64) and R (float), column-major with leading dimension ld.
struct Acc {
    unsigned long long *T = nullptr;
    float *R = nullptr;
    int64_t ld = 0;
};

// Exact levels of the kernel gemm() uses for A and B: T is returned in units of
// 2^-8(exact - 1).  5 for 64-row column tiles, 4 for 7 x 7 slices, 2 for 2 x 2, else 3.
int exact_levels(const Operand &A, const Operand &B);

// Launch C += A B^T (A: M x K, B: N x K) into acc.  Supported: 4 or 5 slices
// per operand and 2 x 2 or 3 x 3 with B.tile_rows 112, 4 x 4, 5 x 4 or 5 x 5 with
// 128, 5 x 5 with 64, 7 x 7 with 96.  An operand stored with more slices can be
// passed with a smaller S: its leading slices are the value rounded to 8 S - 1 bits.
// lower_only: only output tiles with column tile <= row tile (symmetric results,
// requires A.tile_rows == B.tile_rows).  err receives a nonzero code if a wait
// in the kernel gave up.
// lmax = 0 forms every slice pair; lmax = 5, 6 or 7 (4 x 5 slices, 112-wide tiles), 6
// (5 x 4 slices, 128-wide tiles), 5 (4 x 4 slices, 128-wide tiles), 6 (5 x 5 slices,
// 128-wide tiles) or 7 (7 x 7 slices,
// 96-wide tiles) drops the pairs s + t > lmax, about 2^-8(lmax-1) of max|A| max|B| per
// product term; slices that take part in no remaining pair are not read.
// skip (optional device flag): when *skip != 0 at run time the launched kernels
// return at once (a step of an iteration that has converged on the device).
int gemm(const Operand &A, const Operand &B, const Acc &acc, bool lower_only, int *err, cudaStream_t s,
         int lmax = 0, const int *skip = nullptr);

// Row scales and slices of a strided matrix: element (r, c) at src[r*sr + c*sc],
// r < rows, c < k.  Src is float or double.  expo and slices of op must be allocated;
// slices padded with zeros.  rowmax is scratch of rows uint64.  skip_diag: the
// entries r == c are taken as 0 (the off-diagonal part of a square matrix).
template <typename T>
int slice_rows(const T *src, int64_t sr, int64_t sc, const Operand &op, unsigned long long *rowmax,
               cudaStream_t s, bool skip_diag = false, const int *skip = nullptr);

}  // namespace split

// Seed of G^-1 for a symmetric positive definite G (spd_inverse.cu): recursive Schur
// complements on the split products above, FP32 Gauss-Jordan and one Newton-Schulz step
// on blocks of up to kSeedBaseRows rows.  Buffers (device): a/b slices and exponents for
// operands of up to m x m (5 slices, 128-row tiles), T/R accumulators of m x m (zero on
// entry, left zero), rowmax (m), the padded float block and Gauss-Jordan scratch for
// kSeedBaseRows rows, base (2 kSeedBaseRows^2 doubles: a block's input and residual),
// err (product waits that gave up) and flag (set when a pivot was not positive).
constexpr int64_t kSeedBaseRows = 1024;
struct SeedWorkspace {
    __nv_bfloat16 *a_slices, *b_slices;
    int32_t *a_expo, *b_expo;
    unsigned long long *T;
    float *R;
    unsigned long long *rowmax;
    float *gp, *gjws;
    double *base;
    int *err, *flag;
};
int spd_inverse_seed(double *X, int64_t ld, int64_t m, double *scratch, const SeedWorkspace &w, cudaStream_t s);

}  // namespace smx
