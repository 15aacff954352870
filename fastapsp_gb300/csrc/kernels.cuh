// kernels.cuh -- device-side types shared by the engine's CUDA kernels.
//
// Distances are 4-byte values of one of two kinds:
//   float     FP32 distances, unreached = 1e8 (the reference's MAXVALUE,
//             fap/utils/parameter.h:26);
//   uint32_t  int32 distances, unreached = 2^30.  Stored values never exceed
//             2^30, so the bits equal the int32 value; sums of two stored
//             values are formed in 32-bit unsigned arithmetic and cannot wrap.
// Non-negative floats order like their bit patterns, so both kinds use the
// integer atomicMin of the SSSP kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fapk {

template <typename T>
struct Dist;

template <>
struct Dist<float> {
  static __host__ __device__ __forceinline__ float inf() { return 1e8f; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ unsigned bits(float a) { return __float_as_uint(a); }
  static __device__ __forceinline__ float from_bits(unsigned b) { return __uint_as_float(b); }
};

template <>
struct Dist<uint32_t> {
  static __host__ __device__ __forceinline__ uint32_t inf() { return 0x40000000u; }
  static __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b) { return a + b; }
  static __device__ __forceinline__ unsigned bits(uint32_t a) { return a; }
  static __device__ __forceinline__ uint32_t from_bits(unsigned b) { return b; }
};

// Error flags written by kernels into the engine's device status word.
enum : unsigned {
  kErrSsspCap = 1u,      // an SSSP batch reached its iteration cap
  kErrBadInput = 2u,     // a kernel saw an index outside its buffers
};

// One (min,+) product segment: C = min(C0, A (x) B) over a rectangular range.
// The output is tiled in 128x128 CTA tiles made of 2x2 blocks of 64x64.  The
// 64-blocks of a tile are picked from a list of block indices, which lets the
// Floyd-Warshall phases skip the pivot block (`row_skip`/`col_skip`) or pin a
// single block (`row_fix`/`col_fix`).
struct MpSegment {
  const void *A;      // A[i][k] = A[i * lda + k]   (i: output row)
  const void *B;      // B[k][j] = B[k * ldb + j]   (j: output column)
  const int32_t *Bp;  // predecessor of B (same indexing, ldbp)
  void *C;            // C[i][j] = C[i * ldc + j]
  int32_t *Cp;        // predecessor of C (ldcp)
  int64_t lda, ldb, ldbp, ldc, ldcp;
  int32_t M, N, K;     // rows < M, cols < N, k < K
  int32_t row_skip;    // 64-block row index left out of the row list (-1: none)
  int32_t col_skip;    // same for columns
  int32_t row_fix;     // >= 0: the row list is this one block
  int32_t col_fix;     // >= 0: the column list is this one block
  int32_t row_skip2;   // a second block left out of the row list (only when > row_skip >= 0)
  int32_t col_skip2;   // same for columns
  int32_t init_from_c; // 1: start from C/Cp (keep on ties); 0: start unreached/-1
  int32_t tiles_x;     // CTA tiles along columns
  int32_t tile_begin;  // first global CTA index of this segment
  int32_t strip_begin; // first global CTA index in the strip form (min-plus)
  // Optional Floyd-Warshall override of the part's own columns (min-plus of
  // a part's inner rows): where col_part[col] == part, the output takes
  // F[row][col_local[col] - local0] (and Fp) instead of the product.
  const int32_t *col_part;  // null: no override
  const int32_t *col_local;
  const void *F;
  const int32_t *Fp;
  int64_t ldf;
  int32_t part, local0;
  // Floyd-Warshall strips: 1 + the index of the matrix's tensor-map pair in
  // the launch's table (0: none, per-thread copies) and the first row of B
  // (the pivot block row) in the matrix.
  int32_t tmap1;
  int32_t b_row0;
};

// FW diagonal-block job: close the 64x64 pivot block of one matrix.
struct FwDiagJob {
  void *D;
  int32_t *P;
  int64_t ld;
  int32_t size;  // matrix size (rows/cols >= size are outside the matrix)
  int32_t block; // pivot block index
  int32_t prev;  // >= 0: the update of round `prev` (pivot block prev) to this
                 // block row and column is applied first (lookahead: the
                 // remaining-tile launch of round prev left them out); -1: none
};

// A strided row-major matrix of 4-byte values.
struct MatRef {
  const void *p;
  int64_t ld;
  int32_t rows, cols;
};

// One batch of up to 32 SSSP sources: lane l of the batch handles source
// src[l]; its distances/predecessors go to row pointers dist_row[l]/pred_row[l]
// given as element offsets into the output arrays.
struct SsspBatch {
  int32_t count;
  int32_t src[32];
  int64_t row_off[32];
};

}  // namespace fapk
