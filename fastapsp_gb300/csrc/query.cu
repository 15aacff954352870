// query.cu -- point-to-point queries on solve() results kept in device
// memory: the distance of (s, t) and the path from s to t rebuilt from the
// predecessor rows.
//
// Reference counterpart: getDistanceP2P / getPathP2P (fap/fap.h:144-145),
// which the reference declares without bodies (fap/fap.cpp:674-680); its
// results live in host vectors.  Here a caller that solved into device rows
// (fap_solve with device buffers) reads single entries and paths without
// copying the n x n rows to the host.  One thread per query follows the
// predecessors of row s from t back to s (at most n steps: a chain that does
// not reach s is reported as bad input), then, when the path fits the
// caller's slots, walks it again writing the vertices from the end.

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

template <typename T>
__global__ void __launch_bounds__(128) query_kernel(QueryArgs a) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.nq) return;
  const int32_t s = a.src[q], t = a.dst[q];
  if (s < 0 || s >= a.n || t < 0 || t >= a.n) {
    atomicOr(a.status, kErrBadInput);
    a.out_len[q] = 0;
    return;
  }
  const int64_t row = (int64_t)a.ed2st[s] * a.n;  // row of s in the solve() layout
  const T d = static_cast<const T *>(a.dist)[row + t];
  static_cast<T *>(a.out_dist)[q] = d;
  if (!(d < Dist<T>::inf())) {
    a.out_len[q] = 0;
    return;
  }
  const int32_t *prow = a.pred + row;
  int32_t len = 1, v = t;
  while (v != s) {
    v = prow[v];
    if (v < 0 || v >= a.n || len > a.n) {  // broken chain: not predecessors of a solve
      atomicOr(a.status, kErrBadInput);
      a.out_len[q] = 0;
      return;
    }
    len++;
  }
  a.out_len[q] = len;
  if (a.out_path == nullptr || len > a.max_len) return;
  int32_t *path = a.out_path + (int64_t)q * a.max_len;
  v = t;
  for (int32_t i = len - 1; i >= 0; i--) {
    path[i] = v;
    v = prow[v];
  }
}

}  // namespace

cudaError_t launch_query(bool f32, const QueryArgs &a, cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((a.nq + 127) / 128);
  ++launch_count();
  if (f32)
    query_kernel<float><<<blocks, 128, 0, st>>>(a);
  else
    query_kernel<uint32_t><<<blocks, 128, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace fapk
