// transform.cu -- gather of each part's dense Floyd-Warshall matrix and the
// scatter of the closed matrix into the part's result rows.
//
// Reference counterparts: MysubMatBuild_path (fap/utils/util_Myalgorithm.h:
// 44-84) and its GPU form LaunchMysubMatBuildKernel with buildFromCSR /
// buildFromSubGraph / setDiagonal (:87-191); MysubMatDecode_path (:236-247)
// and MysubMatDecode_path_kernel (:193-233).  MyMat1Build (:250-285) has no
// counterpart here: the min-plus reads the inner x boundary block of the FW
// matrix in place.
//
// Matrix layout: part p's matrix is ld_p x ld_p (ld_p = size rounded up to the
// 64-wide FW block) in one arena; padding rows/columns hold "unreached" with a
// zero diagonal, which leaves the FW result of the real block unchanged.
// One CTA builds (or scatters) one matrix row.

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

__device__ __forceinline__ int find_part(const int64_t *row_begin, int nparts, int64_t r) {
  int lo = 0, hi = nparts - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (row_begin[mid] <= r) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One row of the part matrix: boundary rows copy the SSSP rows at the part's
// columns; inner rows start unreached and take the part-local CSR entries
// (later entries overwrite earlier ones, as in the reference); the diagonal is
// 0 with predecessor = the vertex itself.
template <typename T, bool PRED>
__global__ void __launch_bounds__(128) build_kernel(BuildArgs a) {
  const int64_t r = blockIdx.x;
  const int p = find_part(a.row_begin, a.nparts, r);
  const PartDesc pd = a.parts[p];
  const int i = (int)(r - a.row_begin[p]);
  const T INF = Dist<T>::inf();
  T *D = static_cast<T *>(a.mat) + pd.mat_off + (int64_t)i * pd.ld;
  int32_t *P = PRED ? a.matp + pd.mat_off + (int64_t)i * pd.ld : nullptr;
  if (i < pd.bdy) {
    const T *src = static_cast<const T *>(a.rows) + pd.row_off + (int64_t)i * a.ldr;
    const int32_t *srcp = PRED ? a.rowsp + pd.row_off + (int64_t)i * a.ldr : nullptr;
    for (int j = threadIdx.x; j < pd.ld; j += blockDim.x) {
      T d = INF;
      int32_t q = -1;
      if (j < pd.sub) {
        const int v = a.st2ed[pd.start + j];
        d = src[v];
        if (PRED) q = srcp[v];
      }
      if (j == i) {
        d = (T)0;
        q = a.st2ed[pd.start + i];
      }
      D[j] = d;
      if (PRED) P[j] = q;
    }
    return;
  }
  for (int j = threadIdx.x; j < pd.ld; j += blockDim.x) {
    D[j] = (j == i) ? (T)0 : INF;
    if (PRED) P[j] = (j == i && i < pd.sub) ? a.st2ed[pd.start + i] : -1;
  }
  if (i >= pd.sub) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int v = a.st2ed[pd.start + i];
    const int gv = a.graph_id[v];
    const T *w = static_cast<const T *>(a.w);
    for (int e = a.ro[v]; e < a.ro[v + 1]; e++) {
      const int nb = a.col[e];
      if (a.graph_id[nb] != gv) continue;
      const int idx = a.ed2st[nb] - pd.start;
      if (idx >= 0 && idx < pd.sub) {
        D[idx] = w[e];
        if (PRED) P[idx] = v;
      }
    }
    D[i] = (T)0;
    if (PRED) P[i] = v;
  }
}

// Scatter of the closed matrix into the boundary rows at the part's columns
// (MysubMatDecode_path for rows [0, bdy)); the inner rows get their part
// columns from the min-plus epilogue.  One CTA per boundary row.
template <typename T, bool PRED>
__global__ void __launch_bounds__(128) decode_kernel(BuildArgs a, T *rows, int32_t *rowsp) {
  const int64_t r = blockIdx.x;
  const int p = find_part(a.dec_begin, a.nparts, r);
  const PartDesc pd = a.parts[p];
  const int i = (int)(r - a.dec_begin[p]);
  if (i >= pd.bdy) return;
  const T *D = static_cast<const T *>(a.mat) + pd.mat_off + (int64_t)i * pd.ld;
  const int32_t *P = PRED ? a.matp + pd.mat_off + (int64_t)i * pd.ld : nullptr;
  T *dst = rows + pd.dec_off + (int64_t)i * a.ldr;
  int32_t *dstp = PRED ? rowsp + pd.dec_off + (int64_t)i * a.ldr : nullptr;
  for (int j = threadIdx.x; j < pd.sub; j += blockDim.x) {
    const int v = a.st2ed[pd.start + j];
    dst[v] = D[j];
    if (PRED) dstp[v] = P[j];
  }
}

}  // namespace

int &launch_count() {
  static thread_local int count = 0;
  return count;
}

cudaError_t launch_build(bool f32, bool pred, const BuildArgs &a, cudaStream_t st) {
  if (a.total_rows <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)a.total_rows;
  if (f32) {
    if (pred) { ++launch_count(); build_kernel<float, true><<<grid, 128, 0, st>>>(a); }
    else { ++launch_count(); build_kernel<float, false><<<grid, 128, 0, st>>>(a); }
  } else {
    if (pred) { ++launch_count(); build_kernel<uint32_t, true><<<grid, 128, 0, st>>>(a); }
    else { ++launch_count(); build_kernel<uint32_t, false><<<grid, 128, 0, st>>>(a); }
  }
  return cudaGetLastError();
}

cudaError_t launch_decode(bool f32, bool pred, const BuildArgs &a, void *rows, int32_t *rowsp,
                          cudaStream_t st) {
  if (a.dec_rows <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)a.dec_rows;
  if (f32) {
    if (pred) { ++launch_count(); decode_kernel<float, true><<<grid, 128, 0, st>>>(a, (float *)rows, rowsp); }
    else { ++launch_count(); decode_kernel<float, false><<<grid, 128, 0, st>>>(a, (float *)rows, rowsp); }
  } else {
    if (pred) { ++launch_count(); decode_kernel<uint32_t, true><<<grid, 128, 0, st>>>(a, (uint32_t *)rows, rowsp); }
    else { ++launch_count(); decode_kernel<uint32_t, false><<<grid, 128, 0, st>>>(a, (uint32_t *)rows, rowsp); }
  }
  return cudaGetLastError();
}

}  // namespace fapk
