// minplus.cu -- (min,+) tile products and the blocked Floyd-Warshall phases.
//
// Reference counterparts: the min-plus product with predecessors
// (min_plus_path_CPU_advanced, fap/kernel/minplus.h:51-65; GPU kernel
// MatrixMulCUDA6_path, fap/kernel/cuda/minplus.cu:32-189) and the blocked
// Floyd-Warshall (floyd_CPU_path, fap/kernel/floyd.h:38-49; GPU kernels
// fw_kernel1 / FW_kernel1A2 / fw_kernel3, fap/kernel/cuda/floyd.cu:26-267).
//
// Design (GB300): one generic CTA tile kernel computes C = min(C0, A (x) B)
// for a 128x128 output tile with 256 threads, 8x8 outputs per thread held in
// registers, k staged through shared memory in chunks of 32 by cp.async with a
// two-stage pipeline.  The argmin is tracked as the chunk-local k of the last
// strict improvement; after each chunk the predecessor is read from the staged
// B-predecessor tile, so the inner loop is add / compare / two selects.  A
// batch of segments (one per matrix or per FW panel) is served by one launch;
// each CTA finds its segment by binary search over the segments' first tile.
//
// Floyd-Warshall over 64-wide pivot blocks uses the same tile kernel for the
// panel and remaining-tile phases: once the pivot block is closed (shortest
// paths through its own vertices, zero diagonal), the row panel is
// D_rr (x) D_rj, the column panel D_ir (x) D_rr and every other tile
// min(D_ij, D_ir (x) D_rj).  Ties keep the current value, so predecessors
// follow P[i][j] = P[k][j] on strict improvement as in the reference.

#include <cuda_runtime.h>
#include <stdint.h>

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
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait_0() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Block index of list entry g when block `skip` is left out of 0..nblocks-1.
__device__ __forceinline__ int list_block(int g, int skip, int fix, int nblocks) {
  if (fix >= 0) return g == 0 ? fix : -1;
  int len = nblocks - ((skip >= 0 && skip < nblocks) ? 1 : 0);
  if (g >= len) return -1;
  return (skip >= 0 && g >= skip) ? g + 1 : g;
}

template <typename T, bool PRED>
__device__ __forceinline__ void load_chunk(MpSmem<T> &sm, int buf, const MpSegment &s,
                                           const int rbase[2], const int cbase[2], int k0) {
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
  // B (and its predecessors): 32 k x 128 columns; threads run along columns.
  {
    const int j = t & 127;
    const int cb = cbase[j >> 6];
    const int col = cb + (j & 63);
    const bool colok = cb >= 0 && col < s.N;
#pragma unroll 4
    for (int it = 0; it < kBK / 2; it++) {
      const int kk = (t >> 7) + 2 * it;
      const int kg = k0 + kk;
      T *dst = &sm.B[buf][kk][j];
      if (colok && kg < s.K) {
        cp_async4(dst, static_cast<const T *>(s.B) + (int64_t)kg * s.ldb + col);
        if (PRED) cp_async4(&sm.Bp[buf][kk][j], s.Bp + (int64_t)kg * s.ldbp + col);
      } else {
        *dst = INF;
        if (PRED) sm.Bp[buf][kk][j] = -1;
      }
    }
  }
}

template <typename T, bool PRED>
__global__ void __launch_bounds__(kThreads, 1)
    mp_tile_kernel(const MpSegment *__restrict__ segs, int nseg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MpSmem<T> &sm = *reinterpret_cast<MpSmem<T> *>(smem_raw);

  // Segment lookup (binary search on tile_begin).
  const int tile = blockIdx.x;
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (segs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
  }
  const MpSegment s = segs[lo];
  const int local = tile - s.tile_begin;
  const int tyt = local / s.tiles_x, txt = local - tyt * s.tiles_x;
  const int nbr = (s.M + kBlk - 1) / kBlk, nbc = (s.N + kBlk - 1) / kBlk;
  int rbase[2], cbase[2];
#pragma unroll
  for (int g = 0; g < 2; g++) {
    int rb = list_block(2 * tyt + g, s.row_skip, s.row_fix, nbr);
    int cb = list_block(2 * txt + g, s.col_skip, s.col_fix, nbc);
    rbase[g] = rb >= 0 ? rb * kBlk : -1;
    cbase[g] = cb >= 0 ? cb * kBlk : -1;
  }

  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const T INF = Dist<T>::inf();

  T acc[8][8];
  int32_t pred[8][8];
  int arg[8][8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int rb = rbase[r >> 2];
    const int row = rb + ty * 4 + (r & 3);
    const bool rok = rb >= 0 && row < s.M;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int cb = cbase[c >> 2];
      const int col = cb + tx * 4 + (c & 3);
      acc[r][c] = INF;
      pred[r][c] = -1;
      arg[r][c] = -1;
      if (s.init_from_c && rok && cb >= 0 && col < s.N) {
        acc[r][c] = static_cast<const T *>(s.C)[(int64_t)row * s.ldc + col];
        if (PRED) pred[r][c] = s.Cp[(int64_t)row * s.ldcp + col];
      }
    }
  }

  const int nchunks = (s.K + kBK - 1) / kBK;
  if (nchunks > 0) load_chunk<T, PRED>(sm, 0, s, rbase, cbase, 0);
  cp_async_commit();
  for (int ch = 0; ch < nchunks; ch++) {
    const int buf = ch & 1;
    if (ch + 1 < nchunks) load_chunk<T, PRED>(sm, buf ^ 1, s, rbase, cbase, (ch + 1) * kBK);
    cp_async_commit();
    cp_async_wait_1();
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < kBK; kk++) {
      T a[8], b[8];
#pragma unroll
      for (int r = 0; r < 8; r++) a[r] = sm.A[buf][(r >> 2) * kBlk + ty * 4 + (r & 3)][kk];
#pragma unroll
      for (int c = 0; c < 8; c++) b[c] = sm.B[buf][kk][(c >> 2) * kBlk + tx * 4 + (c & 3)];
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const T v = Dist<T>::add(a[r], b[c]);
          if (v < acc[r][c]) {
            acc[r][c] = v;
            if (PRED) arg[r][c] = kk;
          }
        }
    }
    if (PRED) {
#pragma unroll
      for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 8; c++)
          if (arg[r][c] >= 0) {
            pred[r][c] = sm.Bp[buf][arg[r][c]][(c >> 2) * kBlk + tx * 4 + (c & 3)];
            arg[r][c] = -1;
          }
    }
    __syncthreads();
  }
  cp_async_wait_0();

#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int rb = rbase[r >> 2];
    const int row = rb + ty * 4 + (r & 3);
    if (rb < 0 || row >= s.M) continue;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int cb = cbase[c >> 2];
      const int col = cb + tx * 4 + (c & 3);
      if (cb < 0 || col >= s.N) continue;
      static_cast<T *>(s.C)[(int64_t)row * s.ldc + col] = acc[r][c];
      if (PRED) s.Cp[(int64_t)row * s.ldcp + col] = pred[r][c];
    }
  }
}

// Closes the 64x64 pivot block of one matrix per CTA: sequential k inside the
// block, 16 elements per thread, one barrier per k.  Row k and column k do not
// change at step k (zero diagonal), so only strictly improved entries are
// written and no second barrier is needed.
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
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  for (int k = 0; k < kBlk; k++) {
    T a[4], b[4];
    int32_t bp[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      a[q] = D[ty * 4 + q][k];
      b[q] = D[k][tx * 4 + q];
      if (PRED) bp[q] = P[k][tx * 4 + q];
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const T v = Dist<T>::add(a[r], b[c]);
        if (v < D[ty * 4 + r][tx * 4 + c]) {
          D[ty * 4 + r][tx * 4 + c] = v;
          if (PRED) P[ty * 4 + r][tx * 4 + c] = bp[c];
        }
      }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < kBlk * kBlk; idx += blockDim.x) {
    const int i = idx >> 6, j = idx & 63;
    const int gi = base + i, gj = base + j;
    if (gi < job.size && gj < job.size) {
      Dg[(int64_t)gi * job.ld + gj] = D[i][j];
      if (PRED) job.P[(int64_t)gi * job.ld + gj] = P[i][j];
    }
  }
}

template <typename T, bool PRED>
cudaError_t launch_mp_t(const MpSegment *d_segs, int nseg, int total_tiles, cudaStream_t st) {
  if (total_tiles <= 0 || nseg <= 0) return cudaSuccess;
  mp_tile_kernel<T, PRED><<<total_tiles, kThreads, sizeof(MpSmem<T>), st>>>(d_segs, nseg);
  return cudaGetLastError();
}

template <typename T, bool PRED>
cudaError_t set_mp_attr() {
  return cudaFuncSetAttribute(mp_tile_kernel<T, PRED>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MpSmem<T>));
}

}  // namespace

cudaError_t launch_minplus_tiles(bool f32, bool pred, const MpSegment *d_segs, int nseg,
                                 int total_tiles, cudaStream_t st) {
  if (f32) return pred ? launch_mp_t<float, true>(d_segs, nseg, total_tiles, st)
                       : launch_mp_t<float, false>(d_segs, nseg, total_tiles, st);
  return pred ? launch_mp_t<uint32_t, true>(d_segs, nseg, total_tiles, st)
              : launch_mp_t<uint32_t, false>(d_segs, nseg, total_tiles, st);
}

cudaError_t launch_fw_diag(bool f32, bool pred, const FwDiagJob *d_jobs, int njobs,
                           cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (f32) {
    if (pred) fw_diag_kernel<float, true><<<njobs, 256, 0, st>>>(d_jobs);
    else fw_diag_kernel<float, false><<<njobs, 256, 0, st>>>(d_jobs);
  } else {
    if (pred) fw_diag_kernel<uint32_t, true><<<njobs, 256, 0, st>>>(d_jobs);
    else fw_diag_kernel<uint32_t, false><<<njobs, 256, 0, st>>>(d_jobs);
  }
  return cudaGetLastError();
}

cudaError_t init_minplus_kernels() {
  cudaError_t e;
  if ((e = set_mp_attr<float, true>()) != cudaSuccess) return e;
  if ((e = set_mp_attr<float, false>()) != cudaSuccess) return e;
  if ((e = set_mp_attr<uint32_t, true>()) != cudaSuccess) return e;
  return set_mp_attr<uint32_t, false>();
}

int minplus_tile_rows() { return kTile; }
int fw_block() { return kBlk; }

}  // namespace fapk
