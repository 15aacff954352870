// minplus.cu -- (min,+) tile products and the blocked Floyd-Warshall phases.
//
// Reference counterparts: the min-plus product with predecessors
// (min_plus_path_CPU_advanced, fap/kernel/minplus.h:51-65; GPU kernel
// MatrixMulCUDA6_path, fap/kernel/cuda/minplus.cu:32-189) and the blocked
// Floyd-Warshall (floyd_CPU_path, fap/kernel/floyd.h:38-49; GPU kernels
// fw_kernel1 / FW_kernel1A2 / fw_kernel3, fap/kernel/cuda/floyd.cu:26-267).
//
// Kernels of this file:
//  - mp_tile_kernel (FP32 and wide int32): the generic tile form.  One CTA
//    computes C = min(C0, A (x) B) for a 128x128 output tile with 256
//    threads, 8x8 outputs per thread in registers, k staged in chunks of 32
//    by cp.async with a two-stage pipeline; the argmin is the chunk-local k
//    of the last strict improvement, resolved against the staged
//    B-predecessor tile after each chunk.  A batch of segments (one per
//    matrix or FW panel) is one launch; each CTA finds its segment by binary
//    search over the segments' first tile.
//  - mp_tile_packed_kernel, mp_strip_kernel, mp_fwstrip_kernel, fw_pivot_kernel
//    (int32 whose finite results stay below 2^24 - 1): packed keys
//    (d << 7) | idx, one DPX __viaddmin_u32 per add-min, which gives the
//    minimum and, on ties, the smallest idx -- the current value (idx 0)
//    first, then the first k.  The strip kernels keep A resident for a strip
//    of column tiles and skip the steps k whose A column or B row has no
//    finite entry in the tile (such a candidate never wins).
//
// Floyd-Warshall over 64-wide pivot blocks: once the pivot block is closed
// (shortest paths through its own vertices, zero diagonal), the row panel is
// D_rr (x) D_rj, the column panel D_ir (x) D_rr and every other tile
// min(D_ij, D_ir (x) D_rj).  Ties keep the current value, so predecessors
// follow P[i][j] = P[k][j] on strict improvement as in the reference.

#include <cooperative_groups.h>
#include <cuda.h>  // CUtensorMap (the type only; maps are encoded on the host)
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

constexpr int kTile = 128;   // CTA tile (rows and columns)
constexpr int kBlk = 64;     // 64-row / 64-column blocks of a tile
constexpr int kBK = 32;      // k chunk staged in shared memory
constexpr int kThreads = 256;
constexpr int kApad = kBK + 1;  // A rows padded against bank conflicts

template <typename T>
struct MpSmem {
  T A[2][kTile][kApad];
  T B[2][kBK][kTile];
  int32_t Bp[2][kBK][kTile];
};

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait_2() { asm volatile("cp.async.wait_group 2;\n" ::); }
__device__ __forceinline__ void cp_async_wait_0() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Bulk tensor copies (TMA): a 2-D box of a tensor map into shared memory,
// completed on an mbarrier whose phase also waits for the expected bytes.
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// One arrival that also expects `bytes` of copies on the barrier's phase.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// Waits for the phase with this parity to complete: false after `polls`
// unsuccessful polls (each poll may suspend the thread for a short while).
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int polls) {
  const unsigned a = smem_u32(bar);
  for (int i = 0; i < polls; i++) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Orders this thread's earlier shared-memory accesses before later bulk
// copies (the async proxy) into the same buffers.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// The tensor map, copied to global memory by the host before the launch,
// made visible to the copy unit.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap *map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(map) : "memory");
}
// Box of `map` at column x, row y (x a multiple of 4 elements of 4 bytes:
// 16-byte aligned) into dst (16-byte aligned shared memory).  Elements
// outside the tensor arrive as zeros.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Block index of list entry g of 0..nblocks-1 without block `skip` (and
// `skip2`, when it is above `skip`), or of the one-block list `fix`; -1 past
// the list.
__device__ __forceinline__ int list_block(int g, int skip, int skip2, int fix, int nblocks) {
  if (fix >= 0) return g == 0 ? fix : -1;
  int b = g;
  if (skip >= 0) {
    if (b >= skip) b++;
    if (skip2 > skip && b >= skip2) b++;
  }
  return b < nblocks ? b : -1;
}

// Length of such a list.
__device__ __forceinline__ int list_len(int skip, int skip2, int fix, int nblocks) {
  if (fix >= 0) return 1;
  int len = nblocks;
  if (skip >= 0 && skip < nblocks) {
    len--;
    if (skip2 > skip && skip2 < nblocks) len--;
  }
  return len;
}

// Stages k-chunk [k0, k0+32) of A (128 rows, 4-byte cp.async into the padded
// rows) and B (128 columns), and of B's predecessors when WITH_BP (16-byte
// cp.async of 4 columns where aligned); entries outside the matrices are
// written directly as "unreached" / -1.
template <typename T, bool WITH_BP, typename SM>
__device__ __forceinline__ void load_chunk(SM &sm, int buf, const MpSegment &s, const int rbase[2],
                                           const int cbase[2], int k0) {
  const int t = threadIdx.x;
  const T INF = Dist<T>::inf();
  // A: 128 rows x 32 k; consecutive threads take consecutive k of one row.
  {
    const int kk = t & 31;
    const int kg = k0 + kk;
#pragma unroll 4
    for (int it = 0; it < kTile / 8; it++) {
      const int m = (t >> 5) + 8 * it;
      const int rb = rbase[m >> 6];
      const int row = rb + (m & 63);
      T *dst = &sm.A[buf][m][kk];
      if (rb >= 0 && row < s.M && kg < s.K) {
        cp_async4(dst, static_cast<const T *>(s.A) + (int64_t)row * s.lda + kg);
      } else {
        *dst = INF;
      }
    }
  }
  // B (and its predecessors): 32 k x 128 columns; a warp takes one row k,
  // 4 consecutive columns a lane (keys_from_values relies on this mapping).
  {
    const int j4 = (t & 31) * 4;
    const int cb = cbase[j4 >> 6];
    const int col = cb + (j4 & 63);
    const bool full = cb >= 0 && col + 3 < s.N;
    const bool vec = full && (s.ldb & 3) == 0 && (reinterpret_cast<uintptr_t>(s.B) & 15) == 0;
    const bool vecp = WITH_BP && full && (s.ldbp & 3) == 0 && (reinterpret_cast<uintptr_t>(s.Bp) & 15) == 0;
#pragma unroll 4
    for (int it = 0; it < kBK / 8; it++) {
      const int kk = (t >> 5) + 8 * it;
      const int kg = k0 + kk;
      T *dst = &sm.B[buf][kk][j4];
      const T *src = static_cast<const T *>(s.B) + (int64_t)kg * s.ldb + col;
      if (kg < s.K && vec) {
        cp_async16(dst, src);
      } else {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (cb >= 0 && col + q < s.N && kg < s.K) cp_async4(dst + q, src + q);
          else dst[q] = INF;
        }
      }
      if constexpr (WITH_BP) {
        int32_t *dp = &sm.Bp[buf][kk][j4];
        const int32_t *sp = s.Bp + (int64_t)kg * s.ldbp + col;
        if (kg < s.K && vecp) {
          cp_async16(dp, sp);
        } else {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            if (cb >= 0 && col + q < s.N && kg < s.K) cp_async4(dp + q, sp + q);
            else dp[q] = -1;
          }
        }
      }
    }
  }
}

// Output tile geometry of one CTA, resolved from its segment.
struct TileGeom {
  int rbase[2], cbase[2];
  int ty, tx;
};

__device__ __forceinline__ const MpSegment &find_segment(const MpSegment *__restrict__ segs,
                                                         int nseg, int tile) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (segs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
  }
  return segs[lo];
}

__device__ __forceinline__ TileGeom tile_geom(const MpSegment &s, int tile) {
  TileGeom g;
  const int local = tile - s.tile_begin;
  const int tyt = local / s.tiles_x, txt = local - tyt * s.tiles_x;
  const int nbr = (s.M + kBlk - 1) / kBlk, nbc = (s.N + kBlk - 1) / kBlk;
#pragma unroll
  for (int i = 0; i < 2; i++) {
    int rb = list_block(2 * tyt + i, s.row_skip, s.row_skip2, s.row_fix, nbr);
    int cb = list_block(2 * txt + i, s.col_skip, s.col_skip2, s.col_fix, nbc);
    g.rbase[i] = rb >= 0 ? rb * kBlk : -1;
    g.cbase[i] = cb >= 0 ? cb * kBlk : -1;
  }
  g.ty = threadIdx.x >> 4;
  g.tx = threadIdx.x & 15;
  return g;
}

__device__ __forceinline__ int out_row(const TileGeom &g, int r) {
  return g.rbase[r >> 2] < 0 ? -1 : g.rbase[r >> 2] + g.ty * 4 + (r & 3);
}
__device__ __forceinline__ int out_col(const TileGeom &g, int c) {
  return g.cbase[c >> 2] < 0 ? -1 : g.cbase[c >> 2] + g.tx * 4 + (c & 3);
}
__device__ __forceinline__ int smem_row(const TileGeom &g, int r) { return (r >> 2) * kBlk + g.ty * 4 + (r & 3); }
__device__ __forceinline__ int smem_col(const TileGeom &g, int c) { return (c >> 2) * kBlk + g.tx * 4 + (c & 3); }

// In-part columns of the inner rows take the part's Floyd-Warshall values
// (the decode of MysubMatDecode_path, util_Myalgorithm.h:236-247, for these
// rows), so the min-plus epilogue writes every column once.
__device__ __forceinline__ bool fw_column(const MpSegment &s, int col, int64_t &off) {
  if (s.col_part == nullptr || s.col_part[col] != s.part) return false;
  off = (int64_t)(s.col_local[col] - s.local0);
  return true;
}

// Whether the output rows allow 16-byte stores of 4 consecutive columns.
// Stores the values of a 64-column row segment held by 16 lanes (4
// consecutive columns a lane; p = this lane's first column) where the row is
// not 16-byte aligned: each lane stores the aligned 16-byte chunk that starts
// inside its quad, completed with the next lane's first values; the ragged
// ends of the segment (lane 0's values before the first boundary, lane 15's
// after the last) go as single stores.  All 32 lanes call it (the values
// move by shuffles within each half-warp); `ok` drops the stores of a row
// outside the matrix.  (A case split on the misalignment, which is the same
// for the whole warp, measured slower than these selects.)
template <typename V>
__device__ __forceinline__ void store_quad_unaligned(V *p, const V v[4], int tx, bool ok) {
  V nx[4];
#pragma unroll
  for (int q = 0; q < 4; q++) nx[q] = __shfl_down_sync(0xffffffffu, v[q], 1, 16);
  if (!ok) return;
  const int o = (int)((reinterpret_cast<uintptr_t>(p) >> 2) & 3);  // the same for the whole segment
  if (o == 0) {
    __stcs(reinterpret_cast<uint4 *>(p), make_uint4((unsigned)v[0], (unsigned)v[1], (unsigned)v[2], (unsigned)v[3]));
    return;
  }
  if (tx < 15) {  // chunk [p + 4 - o, p + 8 - o): v[4 - o .. 3], then nx[0 .. 3 - o]
    const V w0 = o == 1 ? v[3] : o == 2 ? v[2] : v[1];
    const V w1 = o == 1 ? nx[0] : o == 2 ? v[3] : v[2];
    const V w2 = o == 1 ? nx[1] : o == 2 ? nx[0] : v[3];
    const V w3 = o == 1 ? nx[2] : o == 2 ? nx[1] : nx[0];
    __stcs(reinterpret_cast<uint4 *>(p + 4 - o), make_uint4((unsigned)w0, (unsigned)w1, (unsigned)w2, (unsigned)w3));
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (q >= 4 - o) p[q] = v[q];
  }
  if (tx == 0) {
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (q < 4 - o) p[q] = v[q];
  }
}

template <bool PRED>
__device__ __forceinline__ bool vec_stores_ok(const MpSegment &s) {
  bool ok = (s.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(s.C) & 15) == 0;
  if (PRED) ok = ok && (s.ldcp & 3) == 0 && (reinterpret_cast<uintptr_t>(s.Cp) & 15) == 0;
  return ok;
}

// Stores the 4 outputs of columns col0..col0+3 of `row` (those < N), after
// the part-column override; one 16-byte store per array when all 4 are in
// range and the rows are aligned.
template <typename T, bool PRED>
__device__ __forceinline__ void store_quad(const MpSegment &s, int row, int col0, T d[4],
                                           int32_t p[4], bool vec) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    int64_t j;
    if (col0 + q < s.N && fw_column(s, col0 + q, j)) {
      d[q] = static_cast<const T *>(s.F)[(int64_t)row * s.ldf + j];
      if (PRED) p[q] = s.Fp[(int64_t)row * s.ldf + j];
    }
  }
  T *crow = static_cast<T *>(s.C) + (int64_t)row * s.ldc;
  int32_t *prow = PRED ? s.Cp + (int64_t)row * s.ldcp : nullptr;
  if (vec && col0 + 3 < s.N) {
    uint4 dv;
    dv.x = Dist<T>::bits(d[0]);
    dv.y = Dist<T>::bits(d[1]);
    dv.z = Dist<T>::bits(d[2]);
    dv.w = Dist<T>::bits(d[3]);
    *reinterpret_cast<uint4 *>(crow + col0) = dv;
    if (PRED) *reinterpret_cast<int4 *>(prow + col0) = make_int4(p[0], p[1], p[2], p[3]);
    return;
  }
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (col0 + q < s.N) {
      crow[col0 + q] = d[q];
      if (PRED) prow[col0 + q] = p[q];
    }
}

// Wide form (FP32, and int32 outside the packed range).  Distances are kept
// as their bit patterns, which order like the values (non-negative floats and
// the int32 encoding), so one __vibmin_u32 gives both the new minimum and
// whether the current value was kept (ties keep it: strict improvement).  An
// add-min is then add + vibmin + select; the argmin is the chunk-local k of
// the last strict improvement, resolved against the staged predecessor tile
// after each chunk.
template <typename T, bool PRED>
__device__ __forceinline__ void tile_wide(MpSmem<T> &sm, const MpSegment &s, const TileGeom &g) {
  const unsigned INF = Dist<T>::bits(Dist<T>::inf());
  unsigned acc[8][8];
  int32_t pred[8][8];
  int arg[8][8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int row = out_row(g, r);
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int col = out_col(g, c);
      acc[r][c] = INF;
      pred[r][c] = -1;
      arg[r][c] = -1;
      if (s.init_from_c && row >= 0 && row < s.M && col >= 0 && col < s.N) {
        acc[r][c] = static_cast<const unsigned *>(s.C)[(int64_t)row * s.ldc + col];
        if (PRED) pred[r][c] = s.Cp[(int64_t)row * s.ldcp + col];
      }
    }
  }
  const int nchunks = (s.K + kBK - 1) / kBK;
  if (nchunks > 0) load_chunk<T, PRED>(sm, 0, s, g.rbase, g.cbase, 0);
  cp_async_commit();
  for (int ch = 0; ch < nchunks; ch++) {
    const int buf = ch & 1;
    if (ch + 1 < nchunks) load_chunk<T, PRED>(sm, buf ^ 1, s, g.rbase, g.cbase, (ch + 1) * kBK);
    cp_async_commit();
    cp_async_wait_1();
    __syncthreads();
    const int kn = min(kBK, s.K - ch * kBK);  // steps of this chunk (the rest is fill)
#pragma unroll 2
    for (int kk = 0; kk < kn; kk++) {
      T a[8], b[8];
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = sm.A[buf][smem_row(g, r)][kk];
#pragma unroll
      for (int c = 0; c < 8; c++) b[c] = sm.B[buf][kk][smem_col(g, c)];
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const unsigned v = Dist<T>::bits(Dist<T>::add(a[r], b[c]));
          if (PRED) {
            bool keep;
            acc[r][c] = __vibmin_u32(acc[r][c], v, &keep);
            arg[r][c] = keep ? arg[r][c] : kk;
          } else {
            acc[r][c] = min(acc[r][c], v);
          }
        }
    }
    if (PRED) {
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++)
          if (arg[r][c] >= 0) {
            pred[r][c] = sm.Bp[buf][arg[r][c]][smem_col(g, c)];
            arg[r][c] = -1;
          }
    }
    __syncthreads();
  }
  cp_async_wait_0();
  const bool vec = vec_stores_ok<PRED>(s);
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int row = out_row(g, r);
    if (row < 0 || row >= s.M) continue;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (g.cbase[h] < 0) continue;
      const int col0 = g.cbase[h] + g.tx * 4;
      if (col0 >= s.N) continue;
      T d[4];
      int32_t p[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        d[q] = Dist<T>::from_bits(acc[r][h * 4 + q]);
        p[q] = pred[r][h * 4 + q];
      }
      store_quad<T, PRED>(s, row, col0, d, p, vec);
    }
  }
}

// Packed int32 form.  Keys are (min(d, kPackH) << 7) | idx: idx 0 marks the
// value the output held before the product, idx = k+1 the candidate k.  One
// DPX __viaddmin_u32 per add-min then yields the minimum and, on equal
// distances, the smallest idx -- the current value first, then the first k
// -- which is the strict-improvement, ascending-k rule of the reference.  Two
// keys sum to at most (2 * kPackH) << 7 | 127 < 2^32, so nothing wraps, and
// saturation at kPackH commutes with + and min, so the results are exact when
// every finite result stays below kPackH (checked by the caller).  With
// predecessors K <= 127, so the final idx names k* directly and the
// predecessor is read once, in the epilogue, from B's predecessor row k*.
constexpr unsigned kPackH = (1u << 24) - 1;
constexpr unsigned kIdxBits = 7;
constexpr unsigned kIdxMask = (1u << kIdxBits) - 1;
constexpr int kMaxPackedK = 127;

constexpr int kStagedBpRows = 64;  // B-predecessor rows kept in shared memory

struct KeySmem {
  unsigned A[2][kTile][kApad];
  unsigned B[2][kBK][kTile];
  int32_t Bp[kStagedBpRows][kTile];  // rows k of B's predecessors when K <= 64
  int32_t fwcol[kTile];  // FW-matrix column of each tile column of the own part, else -1
};

// Stages B-predecessor rows [k0, k0+32) into Bp[k0..] (not double-buffered:
// every row of the whole K range keeps its own slot); read only after a
// barrier, so any thread mapping does.
__device__ __forceinline__ void load_bp_rows(KeySmem &sm, const MpSegment &s, const int cbase[2],
                                             int k0) {
  const int t = threadIdx.x;
  const int j = t & 127;
  const int cb = cbase[j >> 6];
  const int col = cb + (j & 63);
  const bool colok = cb >= 0 && col < s.N;
#pragma unroll 4
  for (int it = 0; it < kBK / 2; it++) {
    const int kk = (t >> 7) + 2 * it;
    const int kg = k0 + kk;
    int32_t *dst = &sm.Bp[kg][j];
    if (colok && kg < s.K) cp_async4(dst, s.Bp + (int64_t)kg * s.ldbp + col);
    else *dst = -1;
  }
}

// After this thread's copies of a chunk have landed, turns the elements it
// loaded (same index mapping as load_chunk) into keys.
__device__ __forceinline__ void keys_from_values(KeySmem &sm, int buf, int k0) {
  const int t = threadIdx.x;
  {
    const int kk = t & 31;
#pragma unroll 4
    for (int it = 0; it < kTile / 8; it++) {
      const int m = (t >> 5) + 8 * it;
      sm.A[buf][m][kk] = min(sm.A[buf][m][kk], kPackH) << kIdxBits;
    }
  }
  {
    const int j4 = (t & 31) * 4;
#pragma unroll 4
    for (int it = 0; it < kBK / 8; it++) {
      const int kk = (t >> 5) + 8 * it;
      const unsigned idx = ((unsigned)((k0 + kk) & kMaxPackedK) + 1u) & kIdxMask;
      uint4 *p = reinterpret_cast<uint4 *>(&sm.B[buf][kk][j4]);
      uint4 v = *p;
      v.x = (min(v.x, kPackH) << kIdxBits) | idx;
      v.y = (min(v.y, kPackH) << kIdxBits) | idx;
      v.z = (min(v.z, kPackH) << kIdxBits) | idx;
      v.w = (min(v.w, kPackH) << kIdxBits) | idx;
      *p = v;
    }
  }
}

template <bool PRED>
__global__ void __launch_bounds__(kThreads, 2)
    mp_tile_packed_kernel(const MpSegment *__restrict__ segs, int nseg, int tile0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeySmem &sm = *reinterpret_cast<KeySmem *>(smem_raw);
  __shared__ MpSegment seg;
  const int tile = tile0 + blockIdx.x;
  if (threadIdx.x == 0) seg = find_segment(segs, nseg, tile);
  __syncthreads();
  const MpSegment &s = seg;
  const TileGeom g = tile_geom(s, tile);
  unsigned acc[8][8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int row = out_row(g, r);
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int col = out_col(g, c);
      acc[r][c] = kPackH << kIdxBits;
      if (s.init_from_c && row >= 0 && row < s.M && col >= 0 && col < s.N)
        acc[r][c] = min(static_cast<const unsigned *>(s.C)[(int64_t)row * s.ldc + col], kPackH) << kIdxBits;
    }
  }
  // Own-part columns of the tile (min-plus of inner rows): FW column or -1.
  if (threadIdx.x < kTile) {
    const int j = threadIdx.x;
    const int cb = g.cbase[j >> 6];
    const int col = cb + (j & 63);
    int32_t f = -1;
    if (s.col_part != nullptr && cb >= 0 && col < s.N && s.col_part[col] == s.part)
      f = s.col_local[col] - s.local0;
    sm.fwcol[j] = f;
  }
  const int nchunks = (s.K + kBK - 1) / kBK;
  // B's predecessor rows (K <= 64) go to shared memory in their own cp.async
  // group, waited for only before the epilogue, so their latency hides under
  // the DPX loop.  Groups: chunk 0 | predecessor rows | chunk 1 | ...
  const bool stage_bp = PRED && s.K <= kStagedBpRows;
  if (nchunks > 0) load_chunk<uint32_t, false>(sm, 0, s, g.rbase, g.cbase, 0);
  cp_async_commit();
  if (stage_bp) {
    for (int k0 = 0; k0 < s.K; k0 += kBK) load_bp_rows(sm, s, g.cbase, k0);
    cp_async_commit();
  }
  for (int ch = 0; ch < nchunks; ch++) {
    const int buf = ch & 1;
    if (ch + 1 < nchunks) load_chunk<uint32_t, false>(sm, buf ^ 1, s, g.rbase, g.cbase, (ch + 1) * kBK);
    cp_async_commit();
    if (ch == 0 && stage_bp) cp_async_wait_2(); else cp_async_wait_1();
    keys_from_values(sm, buf, ch * kBK);
    __syncthreads();
    const int kn = min(kBK, s.K - ch * kBK);  // steps of this chunk (the rest is fill)
#pragma unroll 2
    for (int kk = 0; kk < kn; kk++) {
      unsigned a[8], b[8];
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = sm.A[buf][smem_row(g, r)][kk];
#pragma unroll
      for (int c = 0; c < 8; c++) b[c] = sm.B[buf][kk][smem_col(g, c)];
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) acc[r][c] = __viaddmin_u32(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
  cp_async_wait_0();
  __syncthreads();  // staged predecessor rows and column flags visible to every thread
  if (s.init_from_c) {
    // Accumulating product (FW phases): idx 0 means the output kept its value,
    // so neither its distance nor its predecessor is stored again.
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int row = out_row(g, r);
      if (row < 0 || row >= s.M) continue;
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int col = out_col(g, c);
        if (col < 0 || col >= s.N) continue;
        const unsigned key = acc[r][c];
        const unsigned idx = key & kIdxMask;
        if (idx == 0) continue;
        static_cast<unsigned *>(s.C)[(int64_t)row * s.ldc + col] = key >> kIdxBits;
        if (PRED)
          s.Cp[(int64_t)row * s.ldcp + col] =
              stage_bp ? sm.Bp[idx - 1][smem_col(g, c)] : s.Bp[(int64_t)(idx - 1) * s.ldbp + col];
      }
    }
    return;
  }
  const bool vec = vec_stores_ok<PRED>(s);
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int row = out_row(g, r);
    if (row < 0 || row >= s.M) continue;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (g.cbase[h] < 0) continue;
      const int col0 = g.cbase[h] + g.tx * 4;
      if (col0 >= s.N) continue;
      unsigned d[4];
      int32_t p[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int col = col0 + q;
        const int sc = smem_col(g, h * 4 + q);
        const unsigned key = acc[r][h * 4 + q];
        const unsigned dist = key >> kIdxBits;
        const unsigned idx = key & kIdxMask;
        d[q] = dist >= kPackH ? Dist<uint32_t>::inf() : dist;
        p[q] = -1;
        if (PRED && col < s.N && dist < kPackH && idx != 0)
          p[q] = stage_bp ? sm.Bp[idx - 1][sc] : s.Bp[(int64_t)(idx - 1) * s.ldbp + col];
        const int fj = sm.fwcol[sc];
        if (fj >= 0) {  // own-part column: the FW value (the decode of this row)
          d[q] = static_cast<const unsigned *>(s.F)[(int64_t)row * s.ldf + fj];
          if (PRED) p[q] = s.Fp[(int64_t)row * s.ldf + fj];
        }
      }
      unsigned *crow = static_cast<unsigned *>(s.C) + (int64_t)row * s.ldc;
      int32_t *prow = PRED ? s.Cp + (int64_t)row * s.ldcp : nullptr;
      if (vec && col0 + 3 < s.N) {  // streaming stores: the rows are not read again here
        __stcs(reinterpret_cast<uint4 *>(crow + col0), make_uint4(d[0], d[1], d[2], d[3]));
        if (PRED) __stcs(reinterpret_cast<int4 *>(prow + col0), make_int4(p[0], p[1], p[2], p[3]));
      } else {
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (col0 + q < s.N) {
            crow[col0 + q] = d[q];
            if (PRED) prow[col0 + q] = p[q];
          }
      }
    }
  }
}

// Strip form of the packed min-plus for products that do not accumulate into
// C (the inner rows of every part) with K <= kStripMaxK.  One CTA owns a
// strip: one 128-row tile of a segment and the TN-column tiles of
// kStripTiles x 128 consecutive columns.  A's 128 x K block is staged once
// per strip (transposed, so that a thread's 8 row operands of one k are two
// 16-byte loads); B's K x TN tiles are double-buffered, so the next tile's
// copy is in flight while the current one is multiplied; B's predecessor
// rows of the tile's active steps, its own-part FW values and the next
// tile's column flags are copied behind the DPX loop.  The part's own
// columns of a tile (the Floyd-Warshall values replace the product there)
// are listed when the tile's column flags land, and the FW values of up to
// kOwnCap of them are staged; further own columns are read from global
// memory in the epilogue.  The descriptor search, the staging of A and the
// pipeline fill of the tile kernel are paid once per strip instead of once
// per tile.  Shared memory (ks = K rounded up to 4):
//   B[2][ks][TN] | Bp[1 + ks][TN] | colp[2][TN] | coll[2][TN] | ownidx[2][TN] |
//   Fst[kOwnCap][128] | Fpst[kOwnCap][128] | A^T[ks][128]
// and, FP32 only, Ar[128][strip_ar_stride(kseg)] (A row-major) |
// Bq[ks / 4][64] (the current tile's B by step group: 16-byte unit (g, col)
// holds steps 4g .. 4g + 3 of column col).
// Row 0 of Bp holds -1, so the predecessor of every output is Bp[idx][col]
// with the key's idx as it is (0 when unreached).
// Work counters of the strip min-plus (diagnostics): [tiles, tiles with no
// active step, add-mins executed (active steps x the tile's 128 x TN
// outputs, summed over tiles)], summed per CTA.
__device__ unsigned long long g_strip_counters[3];

constexpr int kStripTiles = 16;  // a strip spans kStripTiles x 128 columns
constexpr int kStripMaxK = 100;  // largest K of the strip form
constexpr int kOwnCap = 12;
// Segments are launched in classes of K.  K <= 48: 128 x 64 tiles with 8 x
// 4 outputs a thread, three CTAs per SM.  On sparse products most of a
// tile's time is its fixed work (B keys, masks, epilogue), whose latencies
// only more resident warps hide; against 128 x 128 tiles at two CTAs per SM
// it measured 16 % faster on a 65,536-vertex geometric graph.  (Four CTAs per
// SM for K <= 32, at 64 registers a thread, measured no faster.)  K <= 100:
// 128 x 128 tiles with 8 x 8 outputs a thread (twice the add-mins per shared
// load), one CTA per SM either way at that K.
constexpr int kStripClassK[] = {48, kStripMaxK};
constexpr int kStripClassTN[] = {64, 128};
constexpr int kStripClasses = 2;

// Row stride of the FP32 strip kernel's row-major copy of A for kseg
// steps: kseg, or kseg + 4 when kseg / 4 is even, so that the stride in
// 16-byte units is odd.
__host__ __device__ constexpr int strip_ar_stride(int kseg) { return ((kseg >> 2) & 1) ? kseg : kseg + 4; }

// Shared memory of the strip kernel with TN-column tiles, in bytes; F32 adds
// the row-major copy of A ([128][ks + 4] at most) and the step-group copy
// of B ([ks / 4][64] 16-byte units, within [64][ks + 4] words).
template <int TN, bool F32 = false>
__host__ __device__ constexpr size_t strip_smem_bytes(int ks) {
  return ((size_t)2 * ks * TN + (size_t)(ks + 1) * TN + 6 * TN + (size_t)2 * kOwnCap * kTile +
          (size_t)ks * kTile + (F32 ? (size_t)(kTile + TN) * (ks + 4) : 0)) * 4;
}

__device__ __forceinline__ const MpSegment &find_strip_segment(const MpSegment *__restrict__ segs,
                                                               int nseg, int strip) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (segs[mid].strip_begin <= strip) lo = mid; else hi = mid - 1;
  }
  return segs[lo];
}

// Layout of the FP32 strip kernels' operands in shared memory: entry (k, m)
// of A^T and entry (k, col) of B sit at row k, position m ^ swz(k) and
// col ^ swz(k) -- the 4-entry chunks of step group k / 4 permuted by XOR with
// its low three bits.  Within a group the permutation is the same, so a
// thread's four consecutive rows or columns stay one aligned 16-byte chunk;
// after the add-mins, threads that look up entries of different step groups
// of the same rows or columns hit different banks.  The packed form keeps
// the plain layout (SWZ false).
template <bool SWZ>
__device__ __forceinline__ int swz(int k) {
  return SWZ ? ((k >> 2) & 7) << 2 : 0;
}

// Copies a ks x TN tile of a row-major 4-byte matrix (rows < K, columns
// [col0, col0 + TN) < N) into dst[ks][TN] (SWZ: chunks permuted by swz);
// each thread moves 4 consecutive columns of a row per pass (one 16-byte
// copy when `vec`), and writes `fill` where the source is outside the matrix.
template <int TN, bool SWZ = false>
__device__ __forceinline__ void strip_load_rows(unsigned *dst, const unsigned *src, int64_t ld,
                                                int K, int N, int ks, int col0, bool vec,
                                                unsigned fill) {
  constexpr int TPR = TN / 4;  // threads per row
  const int t = threadIdx.x;
  const int j = (t % TPR) * 4;
  const int col = col0 + j;
  for (int kk = t / TPR; kk < ks; kk += kThreads / TPR) {
    unsigned *d = dst + kk * TN + (j ^ swz<SWZ>(kk));
    const unsigned *g = src + (int64_t)kk * ld + col;
    if (kk < K && vec && col + 3 < N) {
      cp_async16(d, g);
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (kk < K && col + q < N) cp_async4(d + q, g + q);
        else d[q] = fill;
      }
    }
  }
}

// Sets the bits of kmask for the warp's rows of a B tile (two rows of 16
// lanes for TN = 64, starting at lane 0's row kk, which is even; one row for
// TN = 128) that have a finite entry: one ballot and one atomic per warp.
template <int TN>
__device__ __forceinline__ void strip_mark_rows(unsigned *kmask, int kk, bool fin) {
  const unsigned bal = __ballot_sync(0xffffffffu, fin);
  if ((threadIdx.x & 31) == 0) {  // lane 0 holds the warp's first (even) row
    const unsigned bits = TN == 64 ? ((bal & 0xffffu) ? 1u : 0u) | ((bal >> 16) ? 2u : 0u) : (bal ? 1u : 0u);
    if (bits) atomicOr(&kmask[kk >> 5], bits << (kk & 31));
  }
}

// Turns the B values this thread copied (same mapping as strip_load_rows)
// into keys (d << 7) | (k + 1), and sets bit k of kmask (a 128-bit mask in
// shared memory) for every row k that has a finite entry in the tile.
// F32 (TN = 64): the values stay (FP32 bits, "unreached" = the bits of 1e8);
// the row bits are set and the values are also written to Bq, the tile's
// copy by step group (word 4 (g TN + col) + q is step 4g + q of column col).
// ks is a multiple of 4, so a warp's rows are all below ks or all at or past
// it, and the warp's lanes run the loop together.
template <int TN, bool F32 = false>
__device__ __forceinline__ void strip_keys_b(unsigned *Bs, int ks, unsigned *kmask,
                                             unsigned *Bq = nullptr) {
  static_assert(TN == 64 || TN == 128, "row marks assume 16 or 32 lanes a row");
  constexpr int TPR = TN / 4;
  const int t = threadIdx.x;
  const int j = (t % TPR) * 4;
  for (int kk = t / TPR; kk < ks; kk += kThreads / TPR) {
    uint4 *p = reinterpret_cast<uint4 *>(Bs + kk * TN + j);
    const unsigned idx = (unsigned)(kk & kMaxPackedK) + 1u;
    uint4 v = *p;
    if (F32) {
      strip_mark_rows<TN>(kmask, kk, min(min(v.x, v.y), min(v.z, v.w)) < __float_as_uint(Dist<float>::inf()));
      unsigned *q = Bq + ((kk >> 2) * TN + j) * 4 + (kk & 3);
      q[0] = v.x;
      q[4] = v.y;
      q[8] = v.z;
      q[12] = v.w;
      continue;
    }
    const bool fin = min(min(v.x, v.y), min(v.z, v.w)) < kPackH;
    v.x = (min(v.x, kPackH) << kIdxBits) | idx;
    v.y = (min(v.y, kPackH) << kIdxBits) | idx;
    v.z = (min(v.z, kPackH) << kIdxBits) | idx;
    v.w = (min(v.w, kPackH) << kIdxBits) | idx;
    *p = v;
    strip_mark_rows<TN>(kmask, kk, fin);
  }
}

// One add-min of the strip kernel: packed keys (one DPX instruction), or
// FP32 bits with the step idx of the last strict improvement kept in `arg`.
template <bool F32>
__device__ __forceinline__ void strip_addmin(unsigned &acc, int &arg, unsigned a, unsigned b, int idx) {
  if constexpr (F32) {
    const unsigned v = __float_as_uint(__uint_as_float(a) + __uint_as_float(b));
    bool keep;
    acc = __vibmin_u32(acc, v, &keep);
    arg = keep ? arg : idx;
  } else {
    acc = __viaddmin_u32(a, b, acc);
  }
}

// Four add-mins of the FP32 strip kernels, steps k0 .. k0 + 3: the current
// value replaced by the minimum of the four sums when that is below it (a
// strict improvement), and then the group tag (k0 + 1) too.  That leaves the
// step of the last strict improvement in the tagged group: its first step
// whose sum equals the final value, since every earlier step's sum is above
// it (strip_resolve_f32 finds it after the loop).  Four FP32 adds, then
// (MIN3ACC, both strip kernels) two 3-input minimums with the current value
// as an input, a compare and one select, or a 3-input and a 2-input minimum,
// a compare and two selects: one ALU instruction more, but the old and the
// new value are not live together (the min-plus took that form while its
// epilogue still spilled at 128 registers a thread).
template <bool MIN3ACC>
__device__ __forceinline__ void strip_addmin4_f32(unsigned &acc, int &tag, const unsigned a[4],
                                                  const unsigned b[4], int grp) {
  const unsigned v0 = __float_as_uint(__fadd_rn(__uint_as_float(a[0]), __uint_as_float(b[0])));
  const unsigned v1 = __float_as_uint(__fadd_rn(__uint_as_float(a[1]), __uint_as_float(b[1])));
  const unsigned v2 = __float_as_uint(__fadd_rn(__uint_as_float(a[2]), __uint_as_float(b[2])));
  const unsigned v3 = __float_as_uint(__fadd_rn(__uint_as_float(a[3]), __uint_as_float(b[3])));
  if constexpr (MIN3ACC) {
    const unsigned nacc = __vimin3_u32(acc, __vimin3_u32(v0, v1, v2), v3);
    tag = nacc != acc ? grp : tag;
    acc = nacc;
  } else {
    const unsigned t = min(__vimin3_u32(v0, v1, v2), v3);
    const bool imp = t < acc;
    acc = imp ? t : acc;
    tag = imp ? grp : tag;
  }
}

// The step idx (k + 1) of an output whose last strict improvement fell in the
// group tagged `tag` (0: none): the group's first step whose sum has the
// final value's bits.  ap / bp point at the output's A and B entries of the
// group's first step (strides sa, sb between steps).
__device__ __forceinline__ int strip_resolve_f32(unsigned acc, int tag, const unsigned *ap, int sa,
                                                 const unsigned *bp, int sb) {
  const unsigned v0 = __float_as_uint(__fadd_rn(__uint_as_float(ap[0]), __uint_as_float(bp[0])));
  const unsigned v1 = __float_as_uint(__fadd_rn(__uint_as_float(ap[sa]), __uint_as_float(bp[sb])));
  const unsigned v2 = __float_as_uint(__fadd_rn(__uint_as_float(ap[2 * sa]), __uint_as_float(bp[2 * sb])));
  const int j = v0 == acc ? 0 : v1 == acc ? 1 : v2 == acc ? 2 : 3;
  return tag > 0 ? tag + j : 0;
}

// FP32 add-mins of a thread's 8 x 4 outputs over steps [0, kseg) (kseg a
// multiple of 4) in groups of four, then, with PRED, each output's group
// resolved to the step idx (k + 1) of its last strict improvement -- the
// same values and steps as single add-mins in ascending order.  As: A^T
// [k][sa] and Bs: B [k][sb] in the swizzled layout (swz); the thread's rows
// are a0 .. a0 + 3 and a0 + kBlk .. a0 + kBlk + 3, its columns b0 .. b0 + 3.
// With LEAN, the B operands load two columns at a time (24 operands live
// instead of 32).  Without `hi` (uniform over the CTA: the tile's second
// 64-row block is empty) the rows a0 + kBlk .. are left as they are.
template <bool PRED, bool LEAN = false>
__device__ __forceinline__ void addmin_groups_f32(unsigned (&acc)[8][4], int (&arg)[8][4],
                                                  const unsigned *As, int sa, int a0,
                                                  const unsigned *Bs, int sb, int b0, int kseg,
                                                  bool hi = true) {
  for (int kk = 0; kk < kseg; kk += 4) {
    const unsigned *acol = As + kk * sa + (a0 ^ swz<true>(kk));
    const unsigned *bcol = Bs + kk * sb + (b0 ^ swz<true>(kk));
    unsigned b[4][4];  // [column][step]
    if (!LEAN) {
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint4 v = *reinterpret_cast<const uint4 *>(bcol + j * sb);
        b[0][j] = v.x, b[1][j] = v.y, b[2][j] = v.z, b[3][j] = v.w;
      }
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (h == 1 && !hi) break;
      unsigned a[4][4];  // [row of the half][step]
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint4 v = *reinterpret_cast<const uint4 *>(acol + j * sa + h * kBlk);
        a[0][j] = v.x, a[1][j] = v.y, a[2][j] = v.z, a[3][j] = v.w;
      }
#pragma unroll
      for (int ch = 0; ch < 2; ch++) {
        if (LEAN) {
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const uint2 v = *reinterpret_cast<const uint2 *>(bcol + j * sb + ch * 2);
            b[ch * 2][j] = v.x, b[ch * 2 + 1][j] = v.y;
          }
        }
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = ch * 2; c < ch * 2 + 2; c++)
            strip_addmin4_f32<true>(acc[h * 4 + r][c], arg[h * 4 + r][c], a[r], b[c], kk + 1);
      }
    }
  }
  if (PRED) {
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) {
        if (r >= 4 && !hi) continue;
        const int k0 = arg[r][c] > 0 ? arg[r][c] - 1 : 0;
        const int sw = swz<true>(k0);
        arg[r][c] = strip_resolve_f32(acc[r][c], arg[r][c], As + k0 * sa + (a0 ^ sw) + (r >> 2) * kBlk + (r & 3),
                                      sa, Bs + k0 * sb + (b0 ^ sw) + c, sb);
      }
  }
}

// The same for the strip min-plus, from row-major copies of the operands:
// Ar[128][ars] (row m's steps contiguous, ars = strip_ar_stride(kseg)) and
// Bq, the tile's B by step group (16-byte unit g * 64 + col: steps 4g ..
// 4g + 3 of column col).
// One 16-byte load gives a row's or a column's four steps of a group, so the
// resolve takes two loads per output.  Eight consecutive columns of one step
// group are eight consecutive units of Bq, in eight different bank groups,
// and so they stay when the lanes' step groups differ (the resolve); Ar's
// stride is odd in 16-byte units, so the two rows (four apart) that a warp
// reads in the loop lie in different bank groups, and one row's different
// step groups (the resolve) too, up to eight groups apart.  The thread's
// rows are r0 .. r0 + 3 and r0 + 64 .. r0 + 67, its columns tx, tx + 16,
// tx + 32 and tx + 48.  B operands load two columns at a time (24 operands
// live).
template <bool PRED>
__device__ __forceinline__ void addmin_groups_rows_f32(unsigned (&acc)[8][4], int (&arg)[8][4],
                                                       const unsigned *Ar, int ars, int kseg, int r0,
                                                       const unsigned *Bq, int tx) {
  const unsigned *arow = Ar + r0 * ars;  // row r0 + m at arow + m * ars
  const uint4 *bq = reinterpret_cast<const uint4 *>(Bq) + tx;  // (g, tx + 16 c) at bq[g * 64 + 16 c]
  for (int kk = 0; kk < kseg; kk += 4) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      unsigned a[4][4];  // [row of the half][step]
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const uint4 v = *reinterpret_cast<const uint4 *>(arow + (h * kBlk + r) * ars + kk);
        a[r][0] = v.x, a[r][1] = v.y, a[r][2] = v.z, a[r][3] = v.w;
      }
#pragma unroll
      for (int ch = 0; ch < 2; ch++) {
        unsigned b[2][4];  // [column of the pair][step]
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const uint4 v = bq[(kk >> 2) * 64 + (ch * 2 + c) * 16];
          b[c][0] = v.x, b[c][1] = v.y, b[c][2] = v.z, b[c][3] = v.w;
        }
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = 0; c < 2; c++)
            strip_addmin4_f32<true>(acc[h * 4 + r][ch * 2 + c], arg[h * 4 + r][ch * 2 + c], a[r], b[c], kk + 1);
      }
    }
  }
  if (PRED) {
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int tag = arg[r][c];
        const int k0 = tag > 0 ? tag - 1 : 0;
        const uint4 av = *reinterpret_cast<const uint4 *>(arow + ((r >> 2) * kBlk + (r & 3)) * ars + k0);
        const uint4 bv = bq[(k0 >> 2) * 64 + c * 16];
        const unsigned v0 = __float_as_uint(__fadd_rn(__uint_as_float(av.x), __uint_as_float(bv.x)));
        const unsigned v1 = __float_as_uint(__fadd_rn(__uint_as_float(av.y), __uint_as_float(bv.y)));
        const unsigned v2 = __float_as_uint(__fadd_rn(__uint_as_float(av.z), __uint_as_float(bv.z)));
        const unsigned m = acc[r][c];
        const int j = v0 == m ? 0 : v1 == m ? 1 : v2 == m ? 2 : 3;
        arg[r][c] = tag > 0 ? tag + j : 0;
      }
  }
}

// TN = 64 (the class K <= 48): 128x64 tiles, 8x4 outputs per thread, up to
// three CTAs per SM.  TN = 128 (the class K <= 100): 128x128 tiles, 8x8
// outputs per thread, up to two CTAs per SM.
// F32: FP32 distances (any range).  The product keeps each output's value
// bits and the step idx (k + 1, 0 = none) of its last strict improvement in
// two registers: fl(a + b), then __vibmin_u32 for the minimum and whether the
// current value was kept (non-negative floats order like their bits) -- the
// reference's strict-<, ascending-k rule, as in the packed form.  TN = 64
// only, two CTAs per SM.
template <bool PRED, int TN, bool F32 = false, bool UA = false>
__global__ void __launch_bounds__(kThreads, TN == 128 || F32 ? 2 : 3)
    mp_strip_kernel(const MpSegment *__restrict__ segs, int nseg, int ks) {
  constexpr int CH = TN / 64;  // 64-column halves of a thread's outputs
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned *Bs = reinterpret_cast<unsigned *>(smem_raw);  // [2][ks][TN]
  int32_t *Bps = reinterpret_cast<int32_t *>(Bs + 2 * ks * TN);  // [1 + ks][TN]
  int32_t *colp = Bps + (ks + 1) * TN;  // [2][TN] col_part of the tile's columns (per tile parity)
  int32_t *coll = colp + 2 * TN;        // [2][TN] col_local of the tile's columns
  int32_t *ownidx = coll + 2 * TN;      // [2][TN] own column: staging slot, or -2 (not staged); else -1
  unsigned *Fst = reinterpret_cast<unsigned *>(ownidx + 2 * TN);  // [kOwnCap][128 rows]
  int32_t *Fpst = reinterpret_cast<int32_t *>(Fst + kOwnCap * kTile);  // [kOwnCap][128 rows]
  unsigned *As = reinterpret_cast<unsigned *>(Fpst + kOwnCap * kTile);  // A^T [ks][128]
  unsigned *Ar = As + ks * kTile;        // F32: A row-major [128][ars]
  unsigned *Bq = Ar + kTile * (ks + 4);  // F32: the tile's B by step group [ks / 4][64][4]
  __shared__ MpSegment seg;
  __shared__ int s_own[2];                   // own columns of the tile (per tile parity)
  __shared__ int16_t s_ownlist[2][kOwnCap];  // their tile columns, by slot
  __shared__ unsigned s_kmask[2][4];         // rows k of B with a finite entry (per tile parity)
  __shared__ unsigned s_amask[4];            // columns k of A with a finite entry (per strip)
  if (threadIdx.x == 0) {
    seg = find_strip_segment(segs, nseg, blockIdx.x);
    s_own[0] = s_own[1] = 0;
  }
  if (threadIdx.x < 8) (&s_kmask[0][0])[threadIdx.x] = 0u;
  if (threadIdx.x < 4) s_amask[threadIdx.x] = 0u;
  if (threadIdx.x < TN) Bps[threadIdx.x] = -1;  // predecessor of idx 0
  __syncthreads();
  const MpSegment &s = seg;
  const int strips_x = (s.tiles_x + kStripTiles - 1) / kStripTiles;
  const int local = blockIdx.x - s.strip_begin;
  const int rt = local / strips_x;
  // column tiles of TN: this strip's 128-column tiles, split
  const int jt0 = (local - rt * strips_x) * kStripTiles * (128 / TN);
  const int jt1 = min(jt0 + kStripTiles * (128 / TN), (s.N + TN - 1) / TN);
  const int row0 = rt * kTile;
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const unsigned INF = F32 ? __float_as_uint(Dist<float>::inf()) : Dist<uint32_t>::inf();
  const int kseg = (s.K + 3) & ~3;  // this segment's K rounded up to 4 (<= ks)
  const int ars = strip_ar_stride(kseg);  // F32: Ar's row stride
  const bool vec_b = (s.ldb & 3) == 0 && (reinterpret_cast<uintptr_t>(s.B) & 15) == 0;
  const bool vec_bp = PRED && (s.ldbp & 3) == 0 && (reinterpret_cast<uintptr_t>(s.Bp) & 15) == 0;
  const bool vec_c = vec_stores_ok<PRED>(s);
  // The epilogue's view of C in registers (the descriptor is in shared memory,
  // which the compiler reads again after every barrier): this thread's rows
  // are the same for every tile of the strip.
  // (Row offsets within a strip are below 2^31 elements: callers send no
  // leading dimension of 2^24 or more here.)
  const int m_rows = s.M, n_cols = s.N;
  const int ldc = (int)s.ldc, ldcp = (int)s.ldcp;
  unsigned *const c_thr = static_cast<unsigned *>(s.C) + (int64_t)(row0 + ty * 4) * s.ldc;
  int32_t *const p_thr = PRED ? s.Cp + (int64_t)(row0 + ty * 4) * s.ldcp : nullptr;

  auto load_flags = [&](int col0, int fb) {  // column flags of a tile, into parity fb
    if (threadIdx.x < TN) {
      const int j = threadIdx.x, col = col0 + j;
      if (s.col_part != nullptr && col < s.N) {
        cp_async4(&colp[fb * TN + j], s.col_part + col);
        cp_async4(&coll[fb * TN + j], s.col_local + col);
      } else {
        colp[fb * TN + j] = -1;
      }
    }
  };
  // B's predecessor rows of the steps k in (lo, hi) only (row k goes to Bps
  // row k + 1); warp w copies every eighth of them, 4 columns a lane.
  auto load_bp_rows = [&](int col0, unsigned long long lo, unsigned long long hi) {
    const int warp = threadIdx.x >> 5;
    const int j = (threadIdx.x & 31) * 4, col = col0 + j;
    int i = 0;
    while (lo | hi) {
      int k;
      if (lo) {
        k = __ffsll(lo) - 1;
        lo &= lo - 1ull;
      } else {
        k = 64 + __ffsll(hi) - 1;
        hi &= hi - 1ull;
      }
      if ((i++ & 7) == warp && j < TN) {
        int32_t *d = Bps + (k + 1) * TN + j;
        const int32_t *g = s.Bp + (int64_t)k * s.ldbp + col;
        if (vec_bp && col + 3 < s.N) {
          cp_async16(d, g);
        } else {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            if (col + q < s.N) cp_async4(d + q, g + q);
            else d[q] = -1;
          }
        }
      }
    }
  };

  // Prologue: A, B and the column flags of the first tile.  A^T is copied
  // with consecutive threads on consecutive rows (its shared-memory rows are
  // contiguous), the FP32 row-major copy with consecutive threads on
  // consecutive steps of a row (contiguous in both memories).
  for (int idx = threadIdx.x; idx < kTile * kseg; idx += kThreads) {
    const int kk = idx >> 7, m = idx & (kTile - 1);
    unsigned *d = &As[idx];
    if (row0 + m < s.M && kk < s.K)
      cp_async4(d, static_cast<const unsigned *>(s.A) + (int64_t)(row0 + m) * s.lda + kk);
    else
      *d = INF;
    if (F32) {
      const int mr = idx / kseg, kr = idx - mr * kseg;
      unsigned *dr = &Ar[mr * ars + kr];
      if (row0 + mr < s.M && kr < s.K)
        cp_async4(dr, static_cast<const unsigned *>(s.A) + (int64_t)(row0 + mr) * s.lda + kr);
      else
        *dr = INF;
    }
  }
  strip_load_rows<TN>(Bs, static_cast<const unsigned *>(s.B), s.ldb, s.K, s.N, kseg, jt0 * TN, vec_b, INF);
  load_flags(jt0 * TN, 0);
  cp_async_commit();

  // Per tile: two barriers.  (A) after the B keys, masks and own-column list;
  // then the tile's predecessor rows (active steps only), its staged FW
  // values and the next tile's flags are copied (one group), then the next
  // tile's B (a second group), while the add-mins issue; (B) once the first
  // group has landed, before the epilogue.  The next B is waited for at the
  // top of the next tile, so it also has the epilogue to land.  Every buffer
  // written between (A) and (B) was last read before (A); the flags and
  // own-column slots are double-buffered by tile parity because the epilogue
  // of one tile runs into the next tile's list without a barrier.
  unsigned long long n_tiles = 0, n_empty = 0, n_steps = 0;  // work counters (thread 0)
  for (int jt = jt0; jt < jt1; jt++) {
    const int buf = (jt - jt0) & 1;
    unsigned *Bcur = Bs + buf * ks * TN;
    cp_async_wait_0();  // this tile's B (and, first tile, A and the flags)
    if (jt == jt0)  // A keys; a warp converts 32 entries of one step k and marks finite ones
      for (int idx = threadIdx.x; idx < kTile * kseg; idx += kThreads) {
        const unsigned v = As[idx];
        if (!F32) As[idx] = min(v, kPackH) << kIdxBits;
        const int kk = idx >> 7;
        if (__any_sync(0xffffffffu, F32 ? v < INF : v < kPackH) && (threadIdx.x & 31) == 0)
          atomicOr(&s_amask[kk >> 5], 1u << (kk & 31));
      }
    strip_keys_b<TN, F32>(Bcur, kseg, s_kmask[buf], Bq);
    // List the tile's own columns (threads 0..TN-1 copied their column's
    // flags; slots are taken in any order through a counter).
    if (threadIdx.x == 0) s_own[buf ^ 1] = 0;  // used by the next tile
    if (threadIdx.x < 4) s_kmask[buf ^ 1][threadIdx.x] = 0u;
    if (threadIdx.x < TN) {
      const int j = threadIdx.x;
      const bool own = colp[buf * TN + j] == s.part;
      const unsigned bal = __ballot_sync(0xffffffffu, own);
      int base = 0;
      if ((threadIdx.x & 31) == 0 && bal) base = atomicAdd(&s_own[buf], __popc(bal));
      base = __shfl_sync(0xffffffffu, base, 0);
      int slot = -1;
      if (own) {
        slot = base + __popc(bal & ((1u << (threadIdx.x & 31)) - 1u));
        if (slot < kOwnCap) s_ownlist[buf][slot] = (int16_t)j;
        else slot = -2;
      }
      ownidx[buf * TN + j] = slot;
    }
    __syncthreads();  // (A)
    if (jt + 1 < jt1) load_flags((jt + 1) * TN, buf ^ 1);
    const int nown = min(s_own[buf], kOwnCap);
    if (nown > 0) {  // stage the FW values of the own columns (rows of this tile)
      for (int it = threadIdx.x; it < nown * kTile; it += kThreads) {
        const int sl = it / kTile, m = it - sl * kTile;
        if (row0 + m < s.M) {
          const int64_t off =
              (int64_t)(row0 + m) * s.ldf + (coll[buf * TN + s_ownlist[buf][sl]] - s.local0);
          cp_async4(&Fst[sl * kTile + m], static_cast<const unsigned *>(s.F) + off);
          if (PRED) cp_async4(&Fpst[sl * kTile + m], s.Fp + off);
        }
      }
    }
    // Only the steps k whose B row has a finite entry in this tile and whose
    // A column has one in this strip can change an output (any other
    // candidate is at least "unreached", which never wins).
    unsigned long long mlo = (unsigned long long)(s_kmask[buf][0] & s_amask[0]) |
                             ((unsigned long long)(s_kmask[buf][1] & s_amask[1]) << 32);
    unsigned long long mhi = (unsigned long long)(s_kmask[buf][2] & s_amask[2]) |
                             ((unsigned long long)(s_kmask[buf][3] & s_amask[3]) << 32);
    const int nact = __popcll(mlo) + __popcll(mhi);
    n_tiles++;
    n_empty += nact == 0;
    // (FP32 with at least half of the steps active runs all of them)
    n_steps += (unsigned long long)(F32 && CH == 1 && nact > 0 && 2 * nact >= kseg ? kseg : nact) * kTile * TN;
    if (PRED && nact == s.K && s.K > 0)  // every step active: all rows, 16-byte copies spread over the CTA
      strip_load_rows<TN>(reinterpret_cast<unsigned *>(Bps + TN), reinterpret_cast<const unsigned *>(s.Bp),
                          s.ldbp, s.K, s.N, kseg, jt * TN, vec_bp, 0xffffffffu);
    else if (PRED && nact > 0)
      load_bp_rows(jt * TN, mlo, mhi);
    cp_async_commit();
    if (jt + 1 < jt1)  // B[buf ^ 1] was last read by the previous tile's add-mins, before (B)
      strip_load_rows<TN>(Bs + (buf ^ 1) * ks * TN, static_cast<const unsigned *>(s.B), s.ldb, s.K,
                          s.N, kseg, (jt + 1) * TN, vec_b, INF);
    cp_async_commit();

    unsigned acc[8][4 * CH];
    int arg[8][4 * CH];  // F32: step idx of the last strict improvement (0: none)
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4 * CH; c++) {
        acc[r][c] = F32 ? INF : kPackH << kIdxBits;
        arg[r][c] = 0;
      }
    // When every step is active the loop runs over all k (unrolled);
    // otherwise it walks the set bits of the mask -- on graphs with limited
    // reachability most steps are skipped.  Either way the next step's
    // operands load while the current step's add-mins issue.
    {
      // the thread's operands of step k
      auto a_at = [&](int k) { return As + k * kTile + ty * 4; };
      auto b_at = [&](int k) { return Bcur + k * TN + tx * 4; };
      // B operands of step k: four consecutive columns (packed keys), or
      // the FP32 thread's columns tx + 16 c (lanes of a row read
      // consecutive words)
      auto load_b = [&](int k) {
        if (F32) {
          const unsigned *q = Bcur + k * TN + tx;
          return make_uint4(q[0], q[16], q[32], q[48]);
        }
        return *reinterpret_cast<const uint4 *>(b_at(k));
      };
      // FP32 with at least half of the steps active: all steps in groups
      // of four (steps that are not active, or at or past K, hold
      // "unreached" on one side and never win).
      const bool grouped = F32 && CH == 1 && nact > 0 && 2 * nact >= kseg;
      if (grouped) {
        if constexpr (F32 && CH == 1) addmin_groups_rows_f32<PRED>(acc, arg, Ar, ars, kseg, ty * 4, Bq, tx);
      } else if (nact == s.K && s.K > 0) {
        uint4 na0 = *reinterpret_cast<const uint4 *>(a_at(0));
        uint4 na1 = *reinterpret_cast<const uint4 *>(a_at(0) + kBlk);
        uint4 nb0 = load_b(0);
        uint4 nb1 = CH == 2 ? *reinterpret_cast<const uint4 *>(b_at(0) + kBlk) : nb0;
#pragma unroll 2
        for (int kk = 0; kk < kseg; kk++) {
          const unsigned a[8] = {na0.x, na0.y, na0.z, na0.w, na1.x, na1.y, na1.z, na1.w};
          const unsigned b[8] = {nb0.x, nb0.y, nb0.z, nb0.w, nb1.x, nb1.y, nb1.z, nb1.w};
          const int kn = kk + 1 < kseg ? kk + 1 : kk;
          na0 = *reinterpret_cast<const uint4 *>(a_at(kn));
          na1 = *reinterpret_cast<const uint4 *>(a_at(kn) + kBlk);
          nb0 = load_b(kn);
          if (CH == 2) nb1 = *reinterpret_cast<const uint4 *>(b_at(kn) + kBlk);
#pragma unroll
          for (int r = 0; r < 8; r++)
#pragma unroll
            for (int c = 0; c < 4 * CH; c++) strip_addmin<F32>(acc[r][c], arg[r][c], a[r], b[c], kk + 1);
        }
      } else if (nact > 0) {
        auto next_k = [&]() {  // lowest remaining step, or -1
          if (mlo) {
            const int b = __ffsll(mlo) - 1;
            mlo &= mlo - 1ull;
            return b;
          }
          if (mhi) {
            const int b = __ffsll(mhi) - 1;
            mhi &= mhi - 1ull;
            return 64 + b;
          }
          return -1;
        };
        int kk = next_k();
        uint4 na0 = *reinterpret_cast<const uint4 *>(a_at(kk));
        uint4 na1 = *reinterpret_cast<const uint4 *>(a_at(kk) + kBlk);
        uint4 nb0 = load_b(kk);
        uint4 nb1 = CH == 2 ? *reinterpret_cast<const uint4 *>(b_at(kk) + kBlk) : nb0;
        while (kk >= 0) {
          const unsigned a[8] = {na0.x, na0.y, na0.z, na0.w, na1.x, na1.y, na1.z, na1.w};
          const unsigned b[8] = {nb0.x, nb0.y, nb0.z, nb0.w, nb1.x, nb1.y, nb1.z, nb1.w};
          const int cur = kk;
          kk = next_k();
          const int kn = kk >= 0 ? kk : 0;
          na0 = *reinterpret_cast<const uint4 *>(a_at(kn));
          na1 = *reinterpret_cast<const uint4 *>(a_at(kn) + kBlk);
          nb0 = load_b(kn);
          if (CH == 2) nb1 = *reinterpret_cast<const uint4 *>(b_at(kn) + kBlk);
#pragma unroll
          for (int r = 0; r < 8; r++)
#pragma unroll
            for (int c = 0; c < 4 * CH; c++) strip_addmin<F32>(acc[r][c], arg[r][c], a[r], b[c], cur + 1);
        }
      }
    }

    cp_async_wait_1();
    __syncthreads();  // (B)
    // Epilogue: distances, predecessors from the staged rows, own-part
    // columns from the part's Floyd-Warshall matrix (only when the tile has
    // any; the test is uniform over the CTA).
    const int colbase = jt * TN;
    if constexpr (F32) {
      // FP32: the thread's columns are tx + 16 c, so each of the four
      // 4-byte streaming stores of a row writes 64 consecutive bytes per
      // half-warp, whatever the alignment of the row.  The value is at most
      // "unreached"; step idx 0 reads predecessor -1.
      if (nown == 0 && colbase + TN <= n_cols) {  // (uniform) no own column, every column inside
#pragma unroll
        for (int r = 0; r < 8; r++) {
          const int rr = (r >> 2) * kBlk + (r & 3);
          if (row0 + ty * 4 + rr >= m_rows) continue;
          unsigned *cq = c_thr + rr * ldc + colbase + tx;
          int32_t *pq = PRED ? p_thr + rr * ldcp + colbase + tx : nullptr;
#pragma unroll
          for (int c = 0; c < 4; c++) {
            __stcs(cq + 16 * c, acc[r][c]);
            if (PRED) __stcs(pq + 16 * c, Bps[arg[r][c] * TN + tx + 16 * c]);
          }
        }
        continue;
      }
      unsigned ownm = 0;  // bit c: column tx + 16 c is the part's own
      if (nown > 0) {
#pragma unroll
        for (int c = 0; c < 4; c++)
          if (ownidx[buf * TN + tx + 16 * c] != -1) ownm |= 1u << c;
      }
#pragma unroll
      for (int r = 0; r < 8; r++) {
        const int rr = (r >> 2) * kBlk + (r & 3);  // row offset from this thread's first row
        const int row = row0 + ty * 4 + rr;
        if (row >= m_rows) continue;
        unsigned *crow = c_thr + rr * ldc;
        int32_t *prow = PRED ? p_thr + rr * ldcp : nullptr;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int sc = tx + 16 * c, col = colbase + sc;
          unsigned d = acc[r][c];
          int32_t pv = PRED ? Bps[arg[r][c] * TN + sc] : -1;
          if ((ownm >> c) & 1u) {
            const int oi = ownidx[buf * TN + sc];
            if (oi >= 0) {  // own-part column: the FW value, staged
              d = Fst[oi * kTile + row - row0];
              if (PRED) pv = Fpst[oi * kTile + row - row0];
            } else if (oi == -2 && col < n_cols) {  // own-part column beyond the staging slots
              const int64_t fj = coll[buf * TN + sc] - s.local0;
              d = static_cast<const unsigned *>(s.F)[(int64_t)row * s.ldf + fj];
              if (PRED) pv = s.Fp[(int64_t)row * s.ldf + fj];
            }
          }
          if (col < n_cols) {  // streaming stores: the rows are not read again here
            __stcs(crow + col, d);
            if (PRED) __stcs(prow + col, pv);
          }
        }
      }
      continue;
    }
    unsigned ownmask = 0;  // bit h * 4 + q: this thread's column sc0 + q of half h is the part's own
    if (nown > 0) {
#pragma unroll
      for (int c = 0; c < 4 * CH; c++)
        if (ownidx[buf * TN + (c >> 2) * kBlk + tx * 4 + (c & 3)] != -1) ownmask |= 1u << c;
    }
    // The unaligned store form (UA) masks rows and columns outside the
    // matrix per lane instead of skipping them: it moves values between lanes.
    const bool cols_full = colbase + TN <= n_cols;  // uniform over the CTA
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int rr = (r >> 2) * kBlk + (r & 3);  // row offset from this thread's first row
      const int row = row0 + ty * 4 + rr;
      const bool row_ok = row < m_rows;
      if (!UA && !row_ok) continue;
      unsigned *crow = c_thr + rr * ldc;
      int32_t *prow = PRED ? p_thr + rr * ldcp : nullptr;
#pragma unroll
      for (int h = 0; h < CH; h++) {
        const int sc0 = h * kBlk + tx * 4;
        const int col0 = colbase + sc0;
        const bool ok = row_ok && col0 < n_cols;
        if (!UA && !ok) continue;
        unsigned d[4] = {INF, INF, INF, INF};
        int32_t p[4] = {-1, -1, -1, -1};
        // a quad of unreached outputs (the common case on sparse graphs)
        // needs no decode and no predecessor gathers
        const unsigned qmin = min(min(acc[r][h * 4], acc[r][h * 4 + 1]),
                                  min(acc[r][h * 4 + 2], acc[r][h * 4 + 3]));
        if (qmin < (kPackH << kIdxBits)) {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const unsigned key = acc[r][h * 4 + q];
            const unsigned dist = key >> kIdxBits;
            d[q] = dist >= kPackH ? INF : dist;
            if (PRED) p[q] = Bps[(key & kIdxMask) * TN + sc0 + q];
          }
        }
        if ((ownmask >> (h * 4)) & 0xfu) {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            if (!((ownmask >> (h * 4 + q)) & 1u)) continue;
            const int oi = ownidx[buf * TN + sc0 + q];
            if (oi >= 0) {  // own-part column: the FW value, staged
              d[q] = Fst[oi * kTile + row - row0];
              if (PRED) p[q] = Fpst[oi * kTile + row - row0];
            } else if (oi == -2 && ok) {  // own-part column beyond the staging slots
              const int64_t fj = coll[buf * TN + sc0 + q] - s.local0;
              d[q] = static_cast<const unsigned *>(s.F)[(int64_t)row * s.ldf + fj];
              if (PRED) p[q] = s.Fp[(int64_t)row * s.ldf + fj];
            }
          }
        }
        if (vec_c && ok && col0 + 3 < n_cols) {  // streaming stores: the rows are not read again here
          __stcs(reinterpret_cast<uint4 *>(crow + col0), make_uint4(d[0], d[1], d[2], d[3]));
          if (PRED) __stcs(reinterpret_cast<int4 *>(prow + col0), make_int4(p[0], p[1], p[2], p[3]));
        } else if (UA && !vec_c && cols_full) {  // rows not 16-byte aligned: realigned 16-byte stores
          store_quad_unaligned(crow + col0, d, tx, row_ok);
          if (PRED) store_quad_unaligned(prow + col0, p, tx, row_ok);
        } else if (ok) {
#pragma unroll
          for (int q = 0; q < 4; q++)
            if (col0 + q < n_cols) {
              crow[col0 + q] = d[q];
              if (PRED) prow[col0 + q] = p[q];
            }
        }
      }
    }
  }
  cp_async_wait_0();
  if (threadIdx.x == 0 && n_tiles > 0) {
    atomicAdd(&g_strip_counters[0], n_tiles);
    atomicAdd(&g_strip_counters[1], n_empty);
    atomicAdd(&g_strip_counters[2], n_steps);
  }
}

// Strip form of the accumulating packed product of the Floyd-Warshall
// remaining-tile phase: D_ij = min(D_ij, D_ir (x) D_rj) with K <= 64 (one
// pivot block), ties keeping D_ij.  A CTA owns a strip: one 128-row tile of
// the segment's row list (A = D_ir resident) and the column tiles of up to
// kFwStripTiles block pairs of its column list.  Everything a tile needs is
// in flight before it is needed: B (= D_rj) double-buffered, the current
// tile's C and B's predecessors staged behind its DPX loop.  The product starts from "unreached" and C joins in the
// epilogue with index 0, which gives the same minimum and tie rule as
// starting from C.
constexpr int kFwStripTiles = 4;  // block pairs (128 columns) per strip
// Column tile of the form used: one 64-column block (128 x 64 tiles, 8 x 4
// outputs a thread, 112 KB of shared memory, two CTAs per SM, so that one
// CTA's epilogue overlaps the other's add-mins).  TN = 128 (block pairs,
// 197 KB, one CTA per SM) is the other form.
constexpr int kFwStripTN = 64;

template <int TN>
struct FwStripSmem {
  unsigned A[kBlk][kTile];     // A keys, transposed: pivot block x strip rows
  unsigned B[2][kBlk][TN];     // B keys of the current / next tile
  int32_t Bp[kBlk][TN];        // B's predecessors of the current tile
  unsigned C[kTile][TN];       // C of the current tile
};

__device__ __forceinline__ int fw_strips_x(const MpSegment &s) {
  return (s.tiles_x + kFwStripTiles - 1) / kFwStripTiles;
}

// Copies rows [0, 64) of B-like data (row k at src + k * ld, columns of the
// tile's 64-column blocks starting at cbase.x / cbase.y, -1 for none) into
// dst[64][TN] (SWZ: chunks permuted by swz); 16-byte copies of 4 columns
// where aligned, `fill` outside the matrix.
template <int TN, bool SWZ = false>
__device__ __forceinline__ void fw_load_b(unsigned *dst, const unsigned *src, int64_t ld, int K,
                                          int N, int2 cbase, bool vec, unsigned fill) {
  constexpr int TPR = TN / 4;  // threads per row
  const int t = threadIdx.x;
  const int j = (t % TPR) * 4;
  const int cb = (j >> 6) ? cbase.y : cbase.x;
  const int col = cb + (j & 63);
  for (int kk = t / TPR; kk < kBlk; kk += kThreads / TPR) {
    unsigned *d = dst + kk * TN + (j ^ swz<SWZ>(kk));
    const unsigned *g = src + (int64_t)kk * ld + col;
    if (cb >= 0 && kk < K && vec && col + 3 < N) {
      cp_async16(d, g);
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (cb >= 0 && kk < K && col + q < N) cp_async4(d + q, g + q);
        else d[q] = fill;
      }
    }
  }
}

// Work counter of the FW remaining-tile strips (diagnostics): add-mins
// executed (steps run x the tile's 128 x TN outputs), summed per CTA.
__device__ unsigned long long g_fw_counters[1];
// Set when a bulk tensor copy of the FW strips did not complete within its
// poll limit (the kernel then gives up on the strip; the host reports it).
__device__ unsigned g_tma_status;
constexpr int kTmaPolls = 1 << 22;
constexpr unsigned kTmaBox = 64 * 64 * 4;  // bytes of one 64 x 64 box

// F32: FP32 distances (value bits, "unreached" = the bits of 1e8): the
// product keeps each output's value bits and the step (k + 1) of its last
// strict improvement in two registers (the active steps, in order); the
// epilogue stores the product where it is strictly below the current value,
// with the predecessor of that step -- the same result as updating the
// current value step by step.  TN = 64.  (Two steps per pass, as in the
// strip min-plus, measured the same here and spills more.)
// TMA: when the segment's matrix has a tensor-map pair (tmaps[2 (tmap1 - 1)]
// for the distances, + 1 for the predecessors: 64 x 64 boxes of 4-byte
// elements, x = column, y = row), thread 0 stages the tile's C (two boxes),
// B's predecessors and, for packed keys, B itself with bulk tensor copies on
// three mbarriers (the two B buffers, C with the predecessors); the FP32 B
// tile keeps its swizzled layout through per-thread copies.  Without a map
// the per-thread asynchronous copies stage everything.
template <bool PRED, int TN, bool F32 = false>
__global__ void __launch_bounds__(kThreads, TN == 128 ? 1 : 2)
    mp_fwstrip_kernel(const MpSegment *__restrict__ segs, int nseg, const CUtensorMap *__restrict__ tmaps) {
  static_assert(!F32 || TN == 64, "the FP32 form uses 64-column tiles");
  constexpr int CH = TN / 64;   // 64-column blocks of a tile
  constexpr int TPR = TN / 4;   // threads per row in the row-wise copies
  // (a name of its own: the other kernels' dynamic shared memory, under
  // one name, is declared 16-byte aligned; the bulk tensor copies want
  // 128-byte aligned destinations, and B, Bp and C start at multiples of
  // 16 KB of this array)
  extern __shared__ __align__(128) unsigned char fw_smem[];
  FwStripSmem<TN> &sm = *reinterpret_cast<FwStripSmem<TN> *>(fw_smem);
  __shared__ MpSegment seg;
  __shared__ unsigned s_kmask[2][2];  // rows k of B with a finite entry (per tile parity)
  __shared__ unsigned s_amask[2];     // columns k of A with a finite entry (per strip)
  __shared__ __align__(8) unsigned long long s_mbar[3];  // TMA: B buffers 0 and 1; C + B's predecessors
  if (threadIdx.x == 0) {
    seg = find_strip_segment(segs, nseg, blockIdx.x);
    mbar_init(&s_mbar[0], 1);
    mbar_init(&s_mbar[1], 1);
    mbar_init(&s_mbar[2], 1);
    mbar_init_fence();
  }
  if (threadIdx.x < 4) (&s_kmask[0][0])[threadIdx.x] = 0u;
  if (threadIdx.x < 2) s_amask[threadIdx.x] = 0u;
  __syncthreads();
  const MpSegment &s = seg;
  const CUtensorMap *tmap_d = (TN == 64 && tmaps != nullptr && s.tmap1 > 0) ? tmaps + 2 * (s.tmap1 - 1) : nullptr;
  // (uniform over the CTA; the alignment tests only guard the copies' rules:
  // 128-byte shared destinations, 64-byte tensor maps)
  const bool tma = tmap_d != nullptr && (smem_u32(fw_smem) & 127u) == 0 &&
                   (reinterpret_cast<uintptr_t>(tmap_d) & 63) == 0;
  const bool tma_b = tma && !F32;
  if (tma && threadIdx.x == 0) {
    tmap_acquire(tmap_d);
    if (PRED) tmap_acquire(tmap_d + 1);
  }
  const int sx = fw_strips_x(s);
  const int local = blockIdx.x - s.strip_begin;
  const int tyt = local / sx;
  const int nbr = (s.M + kBlk - 1) / kBlk, nbc = (s.N + kBlk - 1) / kBlk;
  // column list length, in blocks, and this strip's column tiles of CH blocks
  const int ncb = list_len(s.col_skip, s.col_skip2, s.col_fix, nbc);
  const int jt0 = (local - tyt * sx) * kFwStripTiles * (2 / CH);
  const int jt1 = min(jt0 + kFwStripTiles * (2 / CH), (ncb + CH - 1) / CH);
  const int rl0 = list_block(2 * tyt, s.row_skip, s.row_skip2, s.row_fix, nbr);
  const int rl1 = list_block(2 * tyt + 1, s.row_skip, s.row_skip2, s.row_fix, nbr);
  const int rbase0 = rl0 >= 0 ? rl0 * kBlk : -1, rbase1 = rl1 >= 0 ? rl1 * kBlk : -1;
  auto col_bases = [&](int jt) {  // first columns of the tile's blocks (-1: none)
    const int b0 = list_block(CH * jt, s.col_skip, s.col_skip2, s.col_fix, nbc);
    const int b1 = CH == 2 ? list_block(CH * jt + 1, s.col_skip, s.col_skip2, s.col_fix, nbc) : -1;
    return make_int2(b0 >= 0 ? b0 * kBlk : -1, b1 >= 0 ? b1 * kBlk : -1);
  };
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const unsigned INF = F32 ? __float_as_uint(Dist<float>::inf()) : Dist<uint32_t>::inf();
  const unsigned FIN = F32 ? INF : kPackH;  // entries below are finite
  const int kseg = (s.K + 3) & ~3;
  const bool vec_b = (s.ldb & 3) == 0 && (reinterpret_cast<uintptr_t>(s.B) & 15) == 0;
  const bool vec_bp = PRED && (s.ldbp & 3) == 0 && (reinterpret_cast<uintptr_t>(s.Bp) & 15) == 0;
  const bool vec_c = (s.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(s.C) & 15) == 0;

  // Prologue: A (transposed) and the first B | the first B's predecessors.
  for (int idx = threadIdx.x; idx < kBlk * kTile; idx += kThreads) {
    const int kk = idx >> 7, m = idx & (kTile - 1);
    const int rb = (m >> 6) ? rbase1 : rbase0;
    const int row = rb + (m & 63);
    unsigned *d = &sm.A[kk][m ^ swz<F32>(kk)];
    if (rb >= 0 && row < s.M && kk < s.K)
      cp_async4(d, static_cast<const unsigned *>(s.A) + (int64_t)row * s.lda + kk);
    else
      *d = INF;
  }
  // B of a tile by TMA (thread 0): one box of pivot rows b_row0.. over the
  // tile's column block, or an arrival without bytes when it has none.
  auto tma_issue_b = [&](int b, int2 c) {
    mbar_expect_tx(&s_mbar[b], c.x >= 0 ? kTmaBox : 0u);
    if (c.x >= 0) tma_load_2d(&sm.B[b][0][0], tmap_d, c.x, s.b_row0, &s_mbar[b]);
  };
  int2 cb = col_bases(jt0);
  if (!tma_b)
    fw_load_b<TN, F32>(&sm.B[0][0][0], static_cast<const unsigned *>(s.B), s.ldb, s.K, s.N, cb, vec_b, INF);
  else if (threadIdx.x == 0)
    tma_issue_b(0, cb);
  cp_async_commit();
  // The epilogue's view of C in registers (the descriptor is in shared memory).
  unsigned *const c_mat = static_cast<unsigned *>(s.C);
  int32_t *const p_mat = s.Cp;
  const int64_t ldc = s.ldc, ldcp = s.ldcp;
  const int m_rows = s.M, n_cols = s.N;
  unsigned long long n_work = 0;  // add-mins executed (thread 0)

  for (int jt = jt0; jt < jt1; jt++) {
    const int buf = (jt - jt0) & 1;
    const unsigned use = (unsigned)(jt - jt0);  // tiles so far: B[buf] is on use >> 1, C on use
    cb = col_bases(jt);
    if (jt + 1 < jt1) {
      if (!tma_b)
        fw_load_b<TN, F32>(&sm.B[buf ^ 1][0][0], static_cast<const unsigned *>(s.B), s.ldb, s.K, s.N,
                  col_bases(jt + 1), vec_b, INF);
      else if (threadIdx.x == 0)
        tma_issue_b(buf ^ 1, col_bases(jt + 1));
    }
    cp_async_commit();
    cp_async_wait_1();  // A and this tile's B have landed
    const bool b_ok = !tma_b || mbar_wait(&s_mbar[buf], (use >> 1) & 1u, kTmaPolls);
    if (jt == jt0)  // A keys; a warp converts 32 entries of one step k and marks finite ones
      for (int idx = threadIdx.x; idx < kBlk * kTile; idx += kThreads) {
        const unsigned v = (&sm.A[0][0])[idx];
        if (!F32) (&sm.A[0][0])[idx] = min(v, kPackH) << kIdxBits;
        const int kk = idx >> 7;
        if (__any_sync(0xffffffffu, v < FIN) && (threadIdx.x & 31) == 0)
          atomicOr(&s_amask[kk >> 5], 1u << (kk & 31));
      }
    {  // B keys; TPR lanes convert a whole row and its first lane marks it when finite
      const int j = (threadIdx.x % TPR) * 4;
      const int lane = threadIdx.x & 31;
      for (int kk = threadIdx.x / TPR; kk < kBlk; kk += kThreads / TPR) {
        uint4 *p = reinterpret_cast<uint4 *>(&sm.B[buf][kk][j]);
        const unsigned idx = (unsigned)kk + 1u;
        uint4 v = *p;
        if (tma_b) {  // steps past K and columns past N: the box brought other rows or zeros
          const int col = cb.x + j;
          const bool row_ok = cb.x >= 0 && kk < s.K;
          if (!row_ok || col >= s.N) v.x = INF;
          if (!row_ok || col + 1 >= s.N) v.y = INF;
          if (!row_ok || col + 2 >= s.N) v.z = INF;
          if (!row_ok || col + 3 >= s.N) v.w = INF;
        }
        const bool fin = min(min(v.x, v.y), min(v.z, v.w)) < FIN;
        if (!F32) {
          v.x = (min(v.x, kPackH) << kIdxBits) | idx;
          v.y = (min(v.y, kPackH) << kIdxBits) | idx;
          v.z = (min(v.z, kPackH) << kIdxBits) | idx;
          v.w = (min(v.w, kPackH) << kIdxBits) | idx;
          *p = v;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, fin);  // every lane runs the same trips
        const unsigned grp = TPR == 32 ? 0xffffffffu : ((1u << (TPR & 31)) - 1u);
        if (lane % TPR == 0 && ((bal >> lane) & grp) != 0u)
          atomicOr(&s_kmask[buf][kk >> 5], 1u << (kk & 31));
      }
      if (threadIdx.x < 2) s_kmask[buf ^ 1][threadIdx.x] = 0u;  // for the next tile
    }
    if (__syncthreads_or(!b_ok)) {  // a B copy never completed: give up on the strip
      if (threadIdx.x == 0) atomicOr(&g_tma_status, 1u);
      mbar_wait(&s_mbar[buf], (use >> 1) & 1u, kTmaPolls);
      if (jt + 1 < jt1) mbar_wait(&s_mbar[buf ^ 1], ((use + 1) >> 1) & 1u, kTmaPolls);
      cp_async_wait_0();
      return;
    }
    // Stage this tile's C behind the DPX loop.
    if (tma) {
      // C's two 64-row boxes and B's predecessors (rows b_row0..), whatever
      // lies outside the matrix arriving as zeros: the epilogue stores no
      // such output and reads only predecessors of steps below K.
      if (threadIdx.x == 0) {
        const bool c0 = cb.x >= 0 && rbase0 >= 0, c1 = cb.x >= 0 && rbase1 >= 0, bp = PRED && cb.x >= 0;
        mbar_expect_tx(&s_mbar[2], (c0 ? kTmaBox : 0u) + (c1 ? kTmaBox : 0u) + (bp ? kTmaBox : 0u));
        if (c0) tma_load_2d(&sm.C[0][0], tmap_d, cb.x, rbase0, &s_mbar[2]);
        if (c1) tma_load_2d(&sm.C[kBlk][0], tmap_d, cb.x, rbase1, &s_mbar[2]);
        if (bp) tma_load_2d(&sm.Bp[0][0], tmap_d + 1, cb.x, s.b_row0, &s_mbar[2]);
      }
    } else {
      const int j = (threadIdx.x % TPR) * 4;
      const int cbj = (j >> 6) ? cb.y : cb.x;
      const int col = cbj + (j & 63);
      for (int m = threadIdx.x / TPR; m < kTile; m += kThreads / TPR) {
        const int rb = (m >> 6) ? rbase1 : rbase0;
        const int row = rb + (m & 63);
        unsigned *d = &sm.C[m][j];
        const unsigned *g = static_cast<const unsigned *>(s.C) + (int64_t)row * s.ldc + col;
        if (rb >= 0 && row < s.M && cbj >= 0 && vec_c && col + 3 < s.N) {
          cp_async16(d, g);
        } else {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            if (rb >= 0 && row < s.M && cbj >= 0 && col + q < s.N) cp_async4(d + q, g + q);
            else d[q] = INF;
          }
        }
      }
      // ... and B's predecessors of this tile, read in the epilogue only
      if (PRED)
        fw_load_b<TN>(reinterpret_cast<unsigned *>(&sm.Bp[0][0]), reinterpret_cast<const unsigned *>(s.Bp),
                      s.ldbp, s.K, s.N, cb, vec_bp, 0xffffffffu);
    }
    cp_async_commit();

    unsigned acc[8][4 * CH];
    int arg[8][4 * CH];  // F32: step (k + 1) of the last strict improvement, 0: none
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int c = 0; c < 4 * CH; c++) {
        acc[r][c] = F32 ? INF : kPackH << kIdxBits;
        arg[r][c] = 0;
      }
    // Only steps k whose B row (pivot row k over this tile's columns) and A
    // column (over this strip's rows) have a finite entry can improve an
    // output: all k (unrolled) when every row
    // has one, else the set bits of the row mask.  The next step's operands
    // load while the current step's add-mins issue.
    {
      const unsigned *acol = &sm.A[0][ty * 4];
      const unsigned *bcol = &sm.B[buf][0][tx * 4];
      unsigned long long msk = (unsigned long long)(s_kmask[buf][0] & s_amask[0]) |
                               ((unsigned long long)(s_kmask[buf][1] & s_amask[1]) << 32);
      if (kseg < 64) msk &= (1ull << kseg) - 1ull;
      const int nact = __popcll(msk);
      // FP32 with at least half of the steps active: all steps in groups of
      // four (steps that are not active hold "unreached" on one side)
      const bool grouped = F32 && CH == 1 && nact > 0 && 2 * nact >= kseg;
      // (the FP32 groups skip the rows of an empty second row block)
      n_work += (unsigned long long)(nact == s.K || grouped ? kseg : nact) * (grouped && rbase1 < 0 ? kBlk : kTile) * TN;
      if (grouped) {
        if constexpr (F32 && CH == 1)
          addmin_groups_f32<PRED>(acc, arg, &sm.A[0][0], kTile, ty * 4, &sm.B[buf][0][0], TN, tx * 4, kseg,
                                  rbase1 >= 0);
      } else if (F32 && msk) {
        while (msk) {  // (the swizzled layout)
          const int kk = __ffsll(msk) - 1;
          msk &= msk - 1ull;
          const unsigned *ak = &sm.A[kk][(ty * 4) ^ swz<true>(kk)];
          const uint4 na0 = *reinterpret_cast<const uint4 *>(ak);
          const uint4 na1 = *reinterpret_cast<const uint4 *>(ak + kBlk);
          const uint4 nb0 = *reinterpret_cast<const uint4 *>(&sm.B[buf][kk][(tx * 4) ^ swz<true>(kk)]);
          const unsigned a[8] = {na0.x, na0.y, na0.z, na0.w, na1.x, na1.y, na1.z, na1.w};
          const unsigned b[4] = {nb0.x, nb0.y, nb0.z, nb0.w};
#pragma unroll
          for (int r = 0; r < 8; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) strip_addmin<true>(acc[r][c], arg[r][c], a[r], b[c], kk + 1);
        }
      } else if (__popcll(msk) == s.K && s.K > 0) {
        uint4 na0 = *reinterpret_cast<const uint4 *>(acol);
        uint4 na1 = *reinterpret_cast<const uint4 *>(acol + kBlk);
        uint4 nb0 = *reinterpret_cast<const uint4 *>(bcol);
        uint4 nb1 = CH == 2 ? *reinterpret_cast<const uint4 *>(bcol + kBlk) : nb0;
#pragma unroll 2
        for (int kk = 0; kk < kseg; kk++) {
          const unsigned a[8] = {na0.x, na0.y, na0.z, na0.w, na1.x, na1.y, na1.z, na1.w};
          const unsigned b[8] = {nb0.x, nb0.y, nb0.z, nb0.w, nb1.x, nb1.y, nb1.z, nb1.w};
          const int kn = kk + 1 < kseg ? kk + 1 : kk;
          na0 = *reinterpret_cast<const uint4 *>(acol + kn * kTile);
          na1 = *reinterpret_cast<const uint4 *>(acol + kn * kTile + kBlk);
          nb0 = *reinterpret_cast<const uint4 *>(bcol + kn * TN);
          if (CH == 2) nb1 = *reinterpret_cast<const uint4 *>(bcol + kn * TN + kBlk);
#pragma unroll
          for (int r = 0; r < 8; r++)
#pragma unroll
            for (int c = 0; c < 4 * CH; c++) acc[r][c] = __viaddmin_u32(a[r], b[c], acc[r][c]);
        }
      } else if (msk) {
        int kk = __ffsll(msk) - 1;
        msk &= msk - 1ull;
        uint4 na0 = *reinterpret_cast<const uint4 *>(acol + kk * kTile);
        uint4 na1 = *reinterpret_cast<const uint4 *>(acol + kk * kTile + kBlk);
        uint4 nb0 = *reinterpret_cast<const uint4 *>(bcol + kk * TN);
        uint4 nb1 = CH == 2 ? *reinterpret_cast<const uint4 *>(bcol + kk * TN + kBlk) : nb0;
        while (kk >= 0) {
          const unsigned a[8] = {na0.x, na0.y, na0.z, na0.w, na1.x, na1.y, na1.z, na1.w};
          const unsigned b[8] = {nb0.x, nb0.y, nb0.z, nb0.w, nb1.x, nb1.y, nb1.z, nb1.w};
          kk = msk ? __ffsll(msk) - 1 : -1;
          if (msk) msk &= msk - 1ull;
          const int kn = kk >= 0 ? kk : 0;
          na0 = *reinterpret_cast<const uint4 *>(acol + kn * kTile);
          na1 = *reinterpret_cast<const uint4 *>(acol + kn * kTile + kBlk);
          nb0 = *reinterpret_cast<const uint4 *>(bcol + kn * TN);
          if (CH == 2) nb1 = *reinterpret_cast<const uint4 *>(bcol + kn * TN + kBlk);
#pragma unroll
          for (int r = 0; r < 8; r++)
#pragma unroll
            for (int c = 0; c < 4 * CH; c++) acc[r][c] = __viaddmin_u32(a[r], b[c], acc[r][c]);
        }
      }
    }
    cp_async_wait_0();
    const bool c_ok = !tma || mbar_wait(&s_mbar[2], use & 1u, kTmaPolls);
    if (__syncthreads_or(!c_ok)) {  // C and the predecessors staged (by every thread, or the copy unit)
      if (threadIdx.x == 0) atomicOr(&g_tma_status, 1u);
      mbar_wait(&s_mbar[2], use & 1u, kTmaPolls);
      if (jt + 1 < jt1 && tma_b) mbar_wait(&s_mbar[buf ^ 1], ((use + 1) >> 1) & 1u, kTmaPolls);
      cp_async_wait_0();
      return;
    }

    // Epilogue: C joins with index 0; only strict improvements are stored.
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int m = (r >> 2) * kBlk + ty * 4 + (r & 3);
      const int rb = (r >> 2) ? rbase1 : rbase0;
      const int row = rb + ty * 4 + (r & 3);
      if (rb < 0 || row >= m_rows) continue;
#pragma unroll
      for (int h = 0; h < CH; h++) {
        const int cbh = h ? cb.y : cb.x;
        if (cbh < 0) continue;
        const int sc0 = h * kBlk + tx * 4;
        const uint4 cv = *reinterpret_cast<const uint4 *>(&sm.C[m][sc0]);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int col = cbh + tx * 4 + q;
          const unsigned cq = q == 0 ? cv.x : q == 1 ? cv.y : q == 2 ? cv.z : cv.w;
          if constexpr (F32) {  // strict improvements only: ties keep the current value
            // (the addresses from the descriptor in shared memory, read
            // again after every barrier: with the register copies the
            // compiler kept the rows' 64-bit offsets live across the tile
            // loop, beside the 64 value and step registers, and spilled)
            if (!(acc[r][h * 4 + q] < cq) || col >= n_cols) continue;
            static_cast<unsigned *>(s.C)[(int64_t)row * s.ldc + col] = acc[r][h * 4 + q];
            if (PRED) s.Cp[(int64_t)row * s.ldcp + col] = sm.Bp[arg[r][h * 4 + q] - 1][sc0 + q];
          } else {
            const unsigned key = min(min(cq, kPackH) << kIdxBits, acc[r][h * 4 + q]);
            const unsigned idx = key & kIdxMask;
            if (idx == 0 || col >= n_cols) continue;
            c_mat[(int64_t)row * ldc + col] = key >> kIdxBits;
            if (PRED) p_mat[(int64_t)row * ldcp + col] = sm.Bp[idx - 1][sc0 + q];
          }
        }
      }
    }
    // C, B[buf] and the predecessors are free again (the fence orders this
    // thread's reads and writes of them before the bulk copies that refill them)
    if (tma) fence_proxy_async_smem();
    __syncthreads();
  }
  cp_async_wait_0();
  if (threadIdx.x == 0 && n_work > 0) atomicAdd(&g_fw_counters[0], n_work);
}

template <typename T, bool PRED>
__global__ void __launch_bounds__(kThreads, 1)
    mp_tile_kernel(const MpSegment *__restrict__ segs, int nseg, int tile0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MpSmem<T> &sm = *reinterpret_cast<MpSmem<T> *>(smem_raw);
  // The segment descriptor stays in shared memory (read where needed) so that
  // the accumulators, argmins and predecessors keep the registers.
  __shared__ MpSegment seg;
  const int tile = tile0 + blockIdx.x;
  if (threadIdx.x == 0) seg = find_segment(segs, nseg, tile);
  __syncthreads();
  const MpSegment &s = seg;
  const TileGeom g = tile_geom(s, tile);
  tile_wide<T, PRED>(sm, s, g);
}

// Largest finite int32 value (< 2^30) of a strided matrix, atomicMax-ed into
// *out; CTAs (blockIdx.x) row-stride over matrix blockIdx.y.
__global__ void max_finite_kernel(const MatRef *__restrict__ mats, unsigned *out) {
  const MatRef mr = mats[blockIdx.y];
  const unsigned *D = static_cast<const unsigned *>(mr.p);
  unsigned m = 0;
  for (int r = blockIdx.x; r < mr.rows; r += gridDim.x)
    for (int c = threadIdx.x; c < mr.cols; c += blockDim.x) {
      const unsigned v = D[(int64_t)r * mr.ld + c];
      if (v < Dist<uint32_t>::inf()) m = max(m, v);
    }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}


// Closes a 64x64 block held in shared memory (D values, P predecessors, row
// pitch 65): sequential k as the reference's floyd_CPU_path
// (fap/kernel/floyd.h:37-48), strict improvements only, P[i][j] = P[k][j].
// Each thread keeps its 4x4 entries in registers; row k and column k do not
// change at step k (zero diagonal), so their owners publish them for the
// next step into a double-buffered row/column copy and one barrier per step
// suffices.  Ends with the closed block back in D/P and a barrier.
template <typename T, bool PRED>
__device__ __forceinline__ void close_block(T (*D)[kBlk + 1], int32_t (*P)[kBlk + 1]) {
  __shared__ T rowk[2][kBlk], colk[2][kBlk];
  __shared__ int32_t prowk[2][kBlk];
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  T d[4][4];
  int32_t p[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      d[i][c] = D[ty * 4 + i][tx * 4 + c];
      p[i][c] = PRED ? P[ty * 4 + i][tx * 4 + c] : -1;
    }
  // publish row 0 / column 0
  if (ty == 0)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      rowk[0][tx * 4 + c] = d[0][c];
      if (PRED) prowk[0][tx * 4 + c] = p[0][c];
    }
  if (tx == 0)
#pragma unroll
    for (int i = 0; i < 4; i++) colk[0][ty * 4 + i] = d[i][0];
  __syncthreads();
  for (int k = 0; k < kBlk; k++) {
    const int buf = k & 1;
    T a[4], b[4];
    int32_t bp[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      a[q] = colk[buf][ty * 4 + q];
      b[q] = rowk[buf][tx * 4 + q];
      if (PRED) bp[q] = prowk[buf][tx * 4 + q];
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const T v = Dist<T>::add(a[i], b[c]);
        if (v < d[i][c]) {
          d[i][c] = v;
          if (PRED) p[i][c] = bp[c];
        }
      }
    const int kn = k + 1;
    if (kn < kBlk) {
      const int kq = kn & 3;
      if (ty == (kn >> 2))
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (i == kq)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              rowk[buf ^ 1][tx * 4 + c] = d[i][c];
              if (PRED) prowk[buf ^ 1][tx * 4 + c] = p[i][c];
            }
      if (tx == (kn >> 2))
#pragma unroll
        for (int c = 0; c < 4; c++)
          if (c == kq)
#pragma unroll
            for (int i = 0; i < 4; i++) colk[buf ^ 1][ty * 4 + i] = d[i][c];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      D[ty * 4 + i][tx * 4 + c] = d[i][c];
      if (PRED) P[ty * 4 + i][tx * 4 + c] = p[i][c];
    }
  __syncthreads();
}

// Closes the 64x64 pivot block of one matrix per CTA (close_block).
template <typename T, bool PRED>
__global__ void __launch_bounds__(256)
    fw_diag_kernel(const FwDiagJob *__restrict__ jobs) {
  __shared__ T D[kBlk][kBlk + 1];
  __shared__ int32_t P[kBlk][kBlk + 1];
  const FwDiagJob job = jobs[blockIdx.x];
  const int base = job.block * kBlk;
  const T INF = Dist<T>::inf();
  T *Dg = static_cast<T *>(job.D);
  for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += blockDim.x) {
    const int i = idx >> 6, j = idx & 63;
    const int gi = base + i, gj = base + j;
    const bool ok = gi < job.size && gj < job.size;
    D[i][j] = ok ? Dg[(int64_t)gi * job.ld + gj] : (i == j ? (T)0 : INF);
    if (PRED) P[i][j] = ok ? job.P[(int64_t)gi * job.ld + gj] : -1;
  }
  __syncthreads();
  close_block<T, PRED>(D, P);
  for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += blockDim.x) {
    const int i = idx >> 6, j = idx & 63;
    const int gi = base + i, gj = base + j;
    if (gi < job.size && gj < job.size) {
      Dg[(int64_t)gi * job.ld + gj] = D[i][j];
      if (PRED) job.P[(int64_t)gi * job.ld + gj] = P[i][j];
    }
  }
}

// Pivot step of one FW round in the packed int32 form, for every matrix of
// the batch: a cluster of kPivotCtas CTAs per matrix (two CTAs per SM).  CTA
// 0 closes the pivot block (as fw_diag_kernel) and writes it back; after a
// cluster barrier the others copy the closed block out of CTA 0's shared
// memory (no second closure, and no read of the block while it is being
// written).  Then CTAs of the first half update the row panel
// D_rb = min(D_rb, D_rr (x) D_rb) and those of the second half the column
// panel D_br = min(D_br, D_br (x) D_rr), each taking every (kPivotCtas/2)-th
// block: 64x64 outputs, 4x4 per thread, packed keys, the block's own values
// joining with index 0.  The panel blocks are a pipeline: the first one's
// copy is issued before the closure (it lands while CTA 0 closes and the
// others wait), each next block's values are copied behind the current
// block's add-mins, and (row panel) its predecessors behind the current
// block's epilogue.  One launch replaces the diagonal launch and the panel
// launch of the tile kernel (whose 128x128 tiles were half empty for 64-wide
// panels).
constexpr int kPivotCtas = 4;

struct PivotSmem {
  unsigned D[kBlk][kBlk + 1];  // pivot block values (closure)
  int32_t P[kBlk][kBlk + 1];   // and predecessors
  unsigned Kp[kBlk][kBlk];     // pivot keys: A^T (row panel) or B (column panel)
  unsigned Xv[kBlk][kBlk];     // the next panel block's values (copy in flight)
  int32_t Xp[kBlk][kBlk];      // the current block's predecessors (row panel)
  unsigned Kx[kBlk][kBlk];     // the current block's keys: B (row panel) or A^T (column panel)
};

// Copies the 64x64 block (rb, cb) of a job's matrix (values, or predecessors
// when P) into dst[64][64], "unreached" / -1 outside the matrix.
template <bool P>
__device__ __forceinline__ void pivot_load_block(unsigned *dst, const FwDiagJob &job, int rb, int cb) {
  const unsigned *src = P ? reinterpret_cast<const unsigned *>(job.P) : static_cast<const unsigned *>(job.D);
  for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += kThreads) {
    const int i = idx >> 6, j = idx & 63;
    const int gi = rb * kBlk + i, gj = cb * kBlk + j;
    if (gi < job.size && gj < job.size) cp_async4(&dst[idx], src + (int64_t)gi * job.ld + gj);
    else dst[idx] = P ? 0xffffffffu : Dist<uint32_t>::inf();
  }
}

// Lookahead part of round `r` of the blocked FW for the 64x64 block (cr, cc)
// of a job's matrix (a block of the next pivot's row or column, or the next
// pivot block itself), which the remaining-tile launch of round r left out:
// C = min(C, A (x) B) with A = block (cr, r), B = block (r, cc), ties keeping
// C, a strict improvement taking B's predecessor -- the same update that
// launch applies to every other tile.  C comes from and goes back to the
// closure buffer sm.D / sm.P (TO_SMEM) or global memory.  Kp, Kx and Xp are
// scratch; ends with a barrier.
template <bool PRED, bool TO_SMEM>
__device__ void pivot_prev_block(PivotSmem &sm, const FwDiagJob &job, int cr, int cc, int r) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  unsigned *Dg = static_cast<unsigned *>(job.D);
  const unsigned INF = Dist<uint32_t>::inf();
  auto inside = [&](int gi, int gj) { return gi < job.size && gj < job.size; };
  unsigned av[4][4], cv[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int li = ty * 4 + i;
    unsigned bv[4];
    int32_t bp[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int lj = tx * 4 + c;
      const int ai = cr * kBlk + li, aj = r * kBlk + lj;
      const int bi = r * kBlk + li, bj = cc * kBlk + lj;
      const int ci = cr * kBlk + li, cj = cc * kBlk + lj;
      av[i][c] = inside(ai, aj) ? Dg[(int64_t)ai * job.ld + aj] : INF;
      bv[c] = inside(bi, bj) ? Dg[(int64_t)bi * job.ld + bj] : INF;
      bp[c] = PRED && inside(bi, bj) ? job.P[(int64_t)bi * job.ld + bj] : -1;
      if (TO_SMEM) cv[i][c] = sm.D[li][lj];
      else cv[i][c] = inside(ci, cj) ? Dg[(int64_t)ci * job.ld + cj] : INF;
    }
    const unsigned id = (unsigned)(li + 1);  // B row k = li
    *reinterpret_cast<uint4 *>(&sm.Kx[li][tx * 4]) =
        make_uint4((min(bv[0], kPackH) << kIdxBits) | id, (min(bv[1], kPackH) << kIdxBits) | id,
                   (min(bv[2], kPackH) << kIdxBits) | id, (min(bv[3], kPackH) << kIdxBits) | id);
    if (PRED) *reinterpret_cast<int4 *>(&sm.Xp[li][tx * 4]) = make_int4(bp[0], bp[1], bp[2], bp[3]);
  }
#pragma unroll
  for (int c = 0; c < 4; c++)  // A^T: k = column of A
    *reinterpret_cast<uint4 *>(&sm.Kp[tx * 4 + c][ty * 4]) =
        make_uint4(min(av[0][c], kPackH) << kIdxBits, min(av[1][c], kPackH) << kIdxBits,
                   min(av[2][c], kPackH) << kIdxBits, min(av[3][c], kPackH) << kIdxBits);
  __syncthreads();
  unsigned acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[i][c] = kPackH << kIdxBits;
#pragma unroll 4
  for (int kk = 0; kk < kBlk; kk++) {
    const uint4 a4 = *reinterpret_cast<const uint4 *>(&sm.Kp[kk][ty * 4]);
    const uint4 b4 = *reinterpret_cast<const uint4 *>(&sm.Kx[kk][tx * 4]);
    const unsigned a[4] = {a4.x, a4.y, a4.z, a4.w};
    const unsigned b[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[i][c] = __viaddmin_u32(a[i], b[c], acc[i][c]);
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int li = ty * 4 + i;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int lj = tx * 4 + c;
      const unsigned key = min(min(cv[i][c], kPackH) << kIdxBits, acc[i][c]);
      const unsigned idx = key & kIdxMask;
      if (idx == 0) continue;
      if (TO_SMEM) {
        sm.D[li][lj] = key >> kIdxBits;
        if (PRED) sm.P[li][lj] = sm.Xp[idx - 1][lj];
      } else {
        const int ci = cr * kBlk + li, cj = cc * kBlk + lj;
        if (!inside(ci, cj)) continue;
        Dg[(int64_t)ci * job.ld + cj] = key >> kIdxBits;
        if (PRED) job.P[(int64_t)ci * job.ld + cj] = sm.Xp[idx - 1][lj];
      }
    }
  }
  __syncthreads();  // scratch free again
}

template <bool PRED>
__global__ void __cluster_dims__(kPivotCtas, 1, 1) __launch_bounds__(kThreads, 2)
    fw_pivot_kernel(const FwDiagJob *__restrict__ jobs) {
  namespace cg = cooperative_groups;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PivotSmem &sm = *reinterpret_cast<PivotSmem *>(smem_raw);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int role = rank / (kPivotCtas / 2);  // 0: row panel, 1: column panel
  const int sub = rank % (kPivotCtas / 2);   // which of the panel's blocks
  constexpr int kStride = kPivotCtas / 2;
  const FwDiagJob job = jobs[blockIdx.x / kPivotCtas];
  const int r = job.block;
  const int nb = (job.size + kBlk - 1) / kBlk;
  const int npanel = nb - 1;
  const unsigned INF = Dist<uint32_t>::inf();
  auto panel_block = [&](int i) { return i < r ? i : i + 1; };  // i-th block other than r
  auto load_values = [&](int pi) {  // panel block pi's values -> Xv
    const int b = panel_block(pi);
    if (role == 0) pivot_load_block<false>(&sm.Xv[0][0], job, r, b);
    else pivot_load_block<false>(&sm.Xv[0][0], job, b, r);
  };
  auto load_preds = [&](int pi) {  // row panel: block pi's predecessors -> Xp
    if (PRED && role == 0)
      pivot_load_block<true>(reinterpret_cast<unsigned *>(&sm.Xp[0][0]), job, r, panel_block(pi));
  };
  // Lookahead: the update of round job.prev to this block row and column
  // (left out by that round's remaining-tile launch) comes first -- CTA 0
  // applies it to the pivot block before the closure, the others to the
  // panel blocks meanwhile.  Without it the first panel block's copy lands
  // during the closure; with it, after the cluster barrier that publishes
  // those updates.
  const int prev = job.prev;
  auto first_copy = [&]() {
    if (sub < npanel) load_values(sub);
    cp_async_commit();
    if (sub < npanel) load_preds(sub);
    cp_async_commit();
  };
  if (prev < 0) first_copy();

  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  if (rank != 0 && prev >= 0) {
    const int lo = min(r, prev), hi = max(r, prev);
    auto other = [&](int t) {  // t-th block other than r and prev
      int b = t;
      if (b >= lo) b++;
      if (b >= hi) b++;
      return b;
    };
    const int nother = nb - 2;
    for (int t = rank - 1; t < 2 * nother; t += kPivotCtas - 1) {
      if (t < nother) pivot_prev_block<PRED, false>(sm, job, r, other(t), prev);
      else pivot_prev_block<PRED, false>(sm, job, other(t - nother), r, prev);
    }
  }
  if (rank == 0) {
    unsigned *Dg = static_cast<unsigned *>(job.D);
    const int base = r * kBlk;
    for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += kThreads) {
      const int i = idx >> 6, j = idx & 63;
      const int gi = base + i, gj = base + j;
      const bool ok = gi < job.size && gj < job.size;
      sm.D[i][j] = ok ? Dg[(int64_t)gi * job.ld + gj] : (i == j ? 0u : INF);
      if (PRED) sm.P[i][j] = ok ? job.P[(int64_t)gi * job.ld + gj] : -1;
    }
    __syncthreads();
    if (prev >= 0) pivot_prev_block<PRED, true>(sm, job, r, r, prev);
    close_block<uint32_t, PRED>(sm.D, sm.P);
    for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += kThreads) {
      const int i = idx >> 6, j = idx & 63;
      const int gi = base + i, gj = base + j;
      if (gi < job.size && gj < job.size) {
        Dg[(int64_t)gi * job.ld + gj] = sm.D[i][j];
        if (PRED) job.P[(int64_t)gi * job.ld + gj] = sm.P[i][j];
      }
    }
  }
  cluster.sync();  // the closed pivot block is in CTA 0's shared memory (and the lookahead updates are in memory)
  if (prev >= 0) first_copy();
  if (rank != 0) {
    const unsigned *rD = cluster.map_shared_rank(&sm.D[0][0], 0);
    const int32_t *rP = cluster.map_shared_rank(&sm.P[0][0], 0);
    for (int idx = threadIdx.x; idx < kBlk * (kBlk + 1); idx += kThreads) {
      (&sm.D[0][0])[idx] = rD[idx];
      if (PRED) (&sm.P[0][0])[idx] = rP[idx];
    }
  }
  cluster.sync();  // CTA 0's shared memory is no longer read; every copy is complete
  for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += kThreads) {
    const int i = idx >> 6, j = idx & 63;
    if (role == 0) sm.Kp[j][i] = min(sm.D[i][j], kPackH) << kIdxBits;  // A^T, idx 0
    else sm.Kp[i][j] = (min(sm.D[i][j], kPackH) << kIdxBits) | (unsigned)(i + 1);  // B, idx k + 1
  }

  for (int pi = sub; pi < npanel; pi += kStride) {
    const int b = panel_block(pi);
    cp_async_wait_1();  // this block's values (its predecessors may still be in flight)
    __syncthreads();    // ... for every thread's part (and Kp, on the first trip)
    // Keys of this block from each thread's own 4x4 outputs, whose values
    // stay in registers for the epilogue.
    unsigned cv[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const uint4 v = *reinterpret_cast<const uint4 *>(&sm.Xv[ty * 4 + i][tx * 4]);
      cv[i][0] = min(v.x, kPackH);
      cv[i][1] = min(v.y, kPackH);
      cv[i][2] = min(v.z, kPackH);
      cv[i][3] = min(v.w, kPackH);
    }
    if (role == 0) {  // B = the block, row k carries idx k + 1
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const unsigned id = (unsigned)(ty * 4 + i + 1);
        *reinterpret_cast<uint4 *>(&sm.Kx[ty * 4 + i][tx * 4]) =
            make_uint4((cv[i][0] << kIdxBits) | id, (cv[i][1] << kIdxBits) | id,
                       (cv[i][2] << kIdxBits) | id, (cv[i][3] << kIdxBits) | id);
      }
    } else {  // A^T of the block
#pragma unroll
      for (int c = 0; c < 4; c++)
        *reinterpret_cast<uint4 *>(&sm.Kx[tx * 4 + c][ty * 4]) =
            make_uint4(cv[0][c] << kIdxBits, cv[1][c] << kIdxBits, cv[2][c] << kIdxBits,
                       cv[3][c] << kIdxBits);
    }
    __syncthreads();  // Kx complete; Xv free for the next block's copy
    if (pi + kStride < npanel) load_values(pi + kStride);
    cp_async_commit();
    const unsigned *Aop = role == 0 ? &sm.Kp[0][0] : &sm.Kx[0][0];
    const unsigned *Bop = role == 0 ? &sm.Kx[0][0] : &sm.Kp[0][0];
    unsigned acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[i][c] = kPackH << kIdxBits;
#pragma unroll 4
    for (int kk = 0; kk < kBlk; kk++) {
      const uint4 av = *reinterpret_cast<const uint4 *>(Aop + kk * kBlk + ty * 4);
      const uint4 bv = *reinterpret_cast<const uint4 *>(Bop + kk * kBlk + tx * 4);
      const unsigned a[4] = {av.x, av.y, av.z, av.w};
      const unsigned bb[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[i][c] = __viaddmin_u32(a[i], bb[c], acc[i][c]);
    }
    cp_async_wait_1();  // this block's predecessors (the next block's values may be in flight)
    __syncthreads();
    unsigned *Dg = static_cast<unsigned *>(job.D);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int li = ty * 4 + i;
      const int gi = (role == 0 ? r : b) * kBlk + li;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int lj = tx * 4 + c;
        const int gj = (role == 0 ? b : r) * kBlk + lj;
        const unsigned key = min(cv[i][c] << kIdxBits, acc[i][c]);
        const unsigned idx = key & kIdxMask;
        if (idx == 0 || gi >= job.size || gj >= job.size) continue;
        Dg[(int64_t)gi * job.ld + gj] = key >> kIdxBits;
        if (PRED) job.P[(int64_t)gi * job.ld + gj] = role == 0 ? sm.Xp[idx - 1][lj] : sm.P[idx - 1][lj];
      }
    }
    __syncthreads();  // Kx and Xp are free again
    if (pi + kStride < npanel) load_preds(pi + kStride);
    cp_async_commit();
  }
  cp_async_wait_0();
}

template <typename T, bool PRED>
cudaError_t launch_mp_t(const MpSegment *d_segs, int nseg, int tiles, int tile0, cudaStream_t st) {
  if (tiles <= 0 || nseg <= 0) return cudaSuccess;
  ++launch_count();
  mp_tile_kernel<T, PRED><<<tiles, kThreads, sizeof(MpSmem<T>), st>>>(d_segs, nseg, tile0);
  return cudaGetLastError();
}

template <bool PRED>
cudaError_t launch_packed_t(const MpSegment *d_segs, int nseg, int tiles, int tile0, cudaStream_t st) {
  if (tiles <= 0 || nseg <= 0) return cudaSuccess;
  ++launch_count();
  mp_tile_packed_kernel<PRED><<<tiles, kThreads, sizeof(KeySmem), st>>>(d_segs, nseg, tile0);
  return cudaGetLastError();
}

template <bool PRED, int TN, bool F32 = false>
cudaError_t launch_strip_t(const MpSegment *d_segs, int nseg, int strips, int ks, cudaStream_t st,
                           bool aligned) {
  if (strips <= 0 || nseg <= 0) return cudaSuccess;
  ++launch_count();
  if (aligned || F32)  // the FP32 epilogue stores 4-byte words at any alignment
    mp_strip_kernel<PRED, TN, F32><<<strips, kThreads, strip_smem_bytes<TN, F32>(ks), st>>>(d_segs, nseg, ks);
  else if constexpr (!F32)
    mp_strip_kernel<PRED, TN, false, true>
        <<<strips, kThreads, strip_smem_bytes<TN, false>(ks), st>>>(d_segs, nseg, ks);
  return cudaGetLastError();
}

template <bool PRED, bool F32>
cudaError_t launch_fwstrip_t(const MpSegment *d_segs, int nseg, int strips, cudaStream_t st,
                             const void *tmaps) {
  if (strips <= 0 || nseg <= 0) return cudaSuccess;
  ++launch_count();
  mp_fwstrip_kernel<PRED, kFwStripTN, F32><<<strips, kThreads, sizeof(FwStripSmem<kFwStripTN>), st>>>(
      d_segs, nseg, static_cast<const CUtensorMap *>(tmaps));
  return cudaGetLastError();
}

template <typename T, bool PRED>
cudaError_t set_mp_attr() {
  return cudaFuncSetAttribute(mp_tile_kernel<T, PRED>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MpSmem<T>));
}

template <bool PRED>
cudaError_t set_packed_attr() {
  return cudaFuncSetAttribute(mp_tile_packed_kernel<PRED>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(KeySmem));
}

}  // namespace

cudaError_t launch_minplus_tiles(bool f32, bool pred, const MpSegment *d_segs, int nseg,
                                 int tiles, bool packed, cudaStream_t st, int tile0) {
  if (f32) return pred ? launch_mp_t<float, true>(d_segs, nseg, tiles, tile0, st)
                       : launch_mp_t<float, false>(d_segs, nseg, tiles, tile0, st);
  if (packed) return pred ? launch_packed_t<true>(d_segs, nseg, tiles, tile0, st)
                          : launch_packed_t<false>(d_segs, nseg, tiles, tile0, st);
  return pred ? launch_mp_t<uint32_t, true>(d_segs, nseg, tiles, tile0, st)
              : launch_mp_t<uint32_t, false>(d_segs, nseg, tiles, tile0, st);
}

cudaError_t launch_minplus_strips(bool pred, const MpSegment *d_segs, int nseg, int strips,
                                  int max_k, cudaStream_t st, bool f32, int tile_cols, bool aligned) {
  if (max_k < 0 || max_k > kStripMaxK) return cudaErrorInvalidValue;
  const int ks = (max_k + 3) & ~3;
  if (f32)  // 128 x 64 tiles at every K (the argmin registers leave no room for 128 x 128)
    return pred ? launch_strip_t<true, 64, true>(d_segs, nseg, strips, ks, st, aligned)
                : launch_strip_t<false, 64, true>(d_segs, nseg, strips, ks, st, aligned);
  const int tn = tile_cols ? tile_cols : kStripClassTN[max_k <= kStripClassK[0] ? 0 : 1];
  if (tn == 64)
    return pred ? launch_strip_t<true, 64>(d_segs, nseg, strips, ks, st, aligned)
                : launch_strip_t<false, 64>(d_segs, nseg, strips, ks, st, aligned);
  if (tn == 128)
    return pred ? launch_strip_t<true, 128>(d_segs, nseg, strips, ks, st, aligned)
                : launch_strip_t<false, 128>(d_segs, nseg, strips, ks, st, aligned);
  return cudaErrorInvalidValue;
}

int minplus_strip_tiles() { return kStripTiles; }

cudaError_t launch_fw_strips(bool pred, const MpSegment *d_segs, int nseg, int strips,
                             cudaStream_t st, bool f32, const void *tmaps) {
  if (f32)
    return pred ? launch_fwstrip_t<true, true>(d_segs, nseg, strips, st, tmaps)
                : launch_fwstrip_t<false, true>(d_segs, nseg, strips, st, tmaps);
  return pred ? launch_fwstrip_t<true, false>(d_segs, nseg, strips, st, tmaps)
              : launch_fwstrip_t<false, false>(d_segs, nseg, strips, st, tmaps);
}

// The driver's tensor-map encoder, looked up once through the runtime (the
// library does not link the driver library itself); null when unavailable.
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      f = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

bool encode_fw_tmaps(void *out, const void *d, const void *p, int64_t ld, int rows, int cols) {
  static_assert(sizeof(CUtensorMap) == 128, "a tensor map is 128 bytes");
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
  if (!enc || !d || rows <= 0 || cols <= 0 || ((ld * 4) & 15) != 0 ||
      (reinterpret_cast<uintptr_t>(d) & 15) != 0 || (p && (reinterpret_cast<uintptr_t>(p) & 15) != 0))
    return false;
  CUtensorMap *m = static_cast<CUtensorMap *>(out);
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {64, 64};
  const cuuint32_t elem[2] = {1, 1};
  for (int i = 0; i < 2; i++) {
    void *base = const_cast<void *>(i == 1 && p ? p : d);
    if (enc(&m[i], CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, base, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

cudaError_t tma_status(unsigned *out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_tma_status, sizeof(unsigned));
  if (e == cudaSuccess && reset && *out) {
    const unsigned zero = 0;
    e = cudaMemcpyToSymbol(g_tma_status, &zero, sizeof(unsigned));
  }
  return e;
}
int fw_strip_tiles() { return kFwStripTiles; }
int minplus_strip_max_k() { return kStripMaxK; }
int minplus_strip_classes() { return kStripClasses; }
int minplus_strip_class_k(int c) { return c >= 0 && c < kStripClasses ? kStripClassK[c] : -1; }
int minplus_strip_class_cols(int c) { return c >= 0 && c < kStripClasses ? kStripClassTN[c] : -1; }

cudaError_t launch_max_finite(const MatRef *d_mats, int nmats, unsigned *out, cudaStream_t st) {
  if (nmats <= 0) return cudaSuccess;
  ++launch_count();
  max_finite_kernel<<<dim3(32, nmats), 256, 0, st>>>(d_mats, out);
  return cudaGetLastError();
}

unsigned pack_limit() { return kPackH; }

cudaError_t fw_strip_counter(unsigned long long *out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_fw_counters, sizeof(unsigned long long));
  if (e != cudaSuccess || !reset) return e;
  const unsigned long long zero = 0;
  return cudaMemcpyToSymbol(g_fw_counters, &zero, sizeof(zero));
}

cudaError_t strip_counters(unsigned long long out[3], bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_strip_counters, sizeof(unsigned long long) * 3);
  if (e != cudaSuccess || !reset) return e;
  const unsigned long long zero[3] = {0, 0, 0};
  return cudaMemcpyToSymbol(g_strip_counters, zero, sizeof(zero));
}
int max_packed_k() { return kMaxPackedK; }

cudaError_t launch_fw_pivot(bool pred, const FwDiagJob *d_jobs, int njobs, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)(kPivotCtas * njobs);
  if (pred) { ++launch_count(); fw_pivot_kernel<true><<<grid, kThreads, sizeof(PivotSmem), st>>>(d_jobs); }
  else { ++launch_count(); fw_pivot_kernel<false><<<grid, kThreads, sizeof(PivotSmem), st>>>(d_jobs); }
  return cudaGetLastError();
}

cudaError_t launch_fw_diag(bool f32, bool pred, const FwDiagJob *d_jobs, int njobs,
                           cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (f32) {
    if (pred) { ++launch_count(); fw_diag_kernel<float, true><<<njobs, 256, 0, st>>>(d_jobs); }
    else { ++launch_count(); fw_diag_kernel<float, false><<<njobs, 256, 0, st>>>(d_jobs); }
  } else {
    if (pred) { ++launch_count(); fw_diag_kernel<uint32_t, true><<<njobs, 256, 0, st>>>(d_jobs); }
    else { ++launch_count(); fw_diag_kernel<uint32_t, false><<<njobs, 256, 0, st>>>(d_jobs); }
  }
  return cudaGetLastError();
}

cudaError_t init_minplus_kernels() {
  cudaError_t e;
  if ((e = set_mp_attr<float, true>()) != cudaSuccess) return e;
  if ((e = set_mp_attr<float, false>()) != cudaSuccess) return e;
  if ((e = set_mp_attr<uint32_t, true>()) != cudaSuccess) return e;
  if ((e = set_mp_attr<uint32_t, false>()) != cudaSuccess) return e;
  if ((e = set_packed_attr<true>()) != cudaSuccess) return e;
  if ((e = set_packed_attr<false>()) != cudaSuccess) return e;
  // either tile width serves any K of the strip form (tile_cols)
  static_assert(kStripClassTN[0] == 64 && kStripClassTN[1] == 128, "strip tile widths");
  const int smax0 = (int)strip_smem_bytes<64>((kStripMaxK + 3) & ~3);
  const int smax1 = (int)strip_smem_bytes<128>((kStripMaxK + 3) & ~3);
#define FAP_STRIP_ATTR1(P, TN, F, UA, SMAX)                                                    \
  if ((e = cudaFuncSetAttribute(mp_strip_kernel<P, TN, F, UA>,                                    \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, SMAX)) != cudaSuccess) \
    return e;
#define FAP_STRIP_ATTR(P, TN, SMAX)  \
  FAP_STRIP_ATTR1(P, TN, false, false, SMAX) \
  FAP_STRIP_ATTR1(P, TN, false, true, SMAX)
  FAP_STRIP_ATTR(true, 64, smax0)
  FAP_STRIP_ATTR(false, 64, smax0)
  FAP_STRIP_ATTR(true, 128, smax1)
  FAP_STRIP_ATTR(false, 128, smax1)
  // FP32: one form for every row alignment
  const int smaxf = (int)strip_smem_bytes<64, true>((kStripMaxK + 3) & ~3);
  FAP_STRIP_ATTR1(true, 64, true, false, smaxf)
  FAP_STRIP_ATTR1(false, 64, true, false, smaxf)
#undef FAP_STRIP_ATTR
#undef FAP_STRIP_ATTR1

  if ((e = cudaFuncSetAttribute(fw_pivot_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(PivotSmem))) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(fw_pivot_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(PivotSmem))) != cudaSuccess)
    return e;
#define FAP_FWSTRIP_ATTR(P, F)                                                           \
  if ((e = cudaFuncSetAttribute(mp_fwstrip_kernel<P, kFwStripTN, F>,                     \
                                cudaFuncAttributeMaxDynamicSharedMemorySize,             \
                                (int)sizeof(FwStripSmem<kFwStripTN>))) != cudaSuccess)   \
    return e;
  FAP_FWSTRIP_ATTR(true, false)
  FAP_FWSTRIP_ATTR(false, false)
  FAP_FWSTRIP_ATTR(true, true)
  FAP_FWSTRIP_ATTR(false, true)
#undef FAP_FWSTRIP_ATTR
  return cudaSuccess;
}

int minplus_tile_rows() { return kTile; }
int fw_block() { return kBlk; }

}  // namespace fapk
