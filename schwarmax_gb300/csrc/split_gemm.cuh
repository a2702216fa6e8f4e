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
//   the remaining levels share one FP32 accumulator whose rounding is 2^-24 of a
//   term already 2^-8 EXACT below the leading one.
// The result for output (i, j) is returned as the exact int64 T and a float R,
// both accumulated with atomics over the k ranges of all CTAs, and the consumer
// forms   C_ij = 2^(eA_i + eB_j - 14) (T_ij 2^-8(EXACT-1) + R_ij)   in double.
// With 4 slices (31 bits) per operand, LMAX = 6 and EXACT = 2 the product error
// is about 2^-31 of max_k |A_ik| sum_k |B_jk| + max_k |B_jk| sum_k |A_ik| plus
// 2^-40 K max_k |A_ik| max_k |B_jk|; 7 slices, LMAX = 8 and EXACT = 4 give
// 2^-55 and 2^-56.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace smx {
namespace split {

constexpr int KT = 32;          // k per pipeline stage (two MMAs of K = 16)
constexpr int MT = 128;         // rows of an A tile (MMA M)
constexpr int OUT_KT = 256;     // k tiles between output flushes at most: 8192 k (int64 running sums)

// bf16 element offset of (row r, column k) inside a rows x KT tile stored as
// 8 x 8 core matrices, core matrix (rg, kg) at ((kg * rows/8) + rg) * 64 elements
__host__ __device__ inline int64_t tile_offset(int r, int k, int rows) {
    return ((int64_t)((k >> 3) * (rows >> 3) + (r >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
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

// Exact levels of the kernel used for (a_slices, b_slices, lmax): T is returned
// in units of 2^-8(exact - 1).  4 for 7 x 7 slices with lmax 8 (about 2^-55),
// else 2.
int exact_levels(int a_slices, int b_slices, int lmax);

// Launch C += A B^T (A: M x K, B: N x K) into acc; B.tile_rows is 112, 128
// (4 or 5 slices, lmax 6) or 96 (7 x 7 slices, lmax 8).
// lower_only: only output tiles with column tile <= row tile (symmetric results,
// requires A.tile_rows == B.tile_rows).  err receives a nonzero code if a wait
// in the kernel gave up.
int gemm(const Operand &A, const Operand &B, int lmax, const Acc &acc, bool lower_only, int *err,
         cudaStream_t s);

// Row scales and slices of a strided matrix: element (r, c) at src[r*sr + c*sc],
// r < rows, c < k.  Src is float or double.  expo and slices of op must be allocated;
// slices padded with zeros.  rowmax is scratch of rows uint64.
template <typename T>
int slice_rows(const T *src, int64_t sr, int64_t sc, const Operand &op, unsigned long long *rowmax,
               cudaStream_t s);

}  // namespace split
}  // namespace smx
