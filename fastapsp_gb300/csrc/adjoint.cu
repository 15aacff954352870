// adjoint.cu -- reverse-mode derivative of shortest-path distances with
// respect to edge weights (no counterpart in the reference).
//
// A shortest-path distance is the sum of the weights along the chosen path,
// so dD[s][t]/dw_e is 1 for every edge on that path and 0 elsewhere (away from
// ties).  Given upstream gradients g for a list of (s, t) pairs, the adjoint
// walks the predecessor path t <- pred[s][t] <- ... <- s recorded by the
// forward pass and adds g to the gradient of each edge it crosses.  One thread
// walks one pair; the walk is capped at the vertex count and flags an error
// instead of looping if the predecessors do not lead back to s.

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

// Graph form: pred rows in solve() layout (row of vertex s = ed2st[s]); the
// edge u->v of a step is the lightest CSR entry u->v (the one a shortest path
// uses), first in CSR order on equal weights.
__global__ void backward_graph_kernel(int32_t n, const int32_t *__restrict__ ro,
                                      const int32_t *__restrict__ col, const float *__restrict__ w,
                                      const int32_t *__restrict__ ed2st,
                                      const int32_t *__restrict__ pred, int32_t npairs,
                                      const int32_t *__restrict__ s, const int32_t *__restrict__ t,
                                      const float *__restrict__ g, float *__restrict__ dw,
                                      unsigned *status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npairs) return;
  const int src = s[i], dst = t[i];
  const float gi = g[i];
  if (src < 0 || src >= n || dst < 0 || dst >= n) {
    atomicOr(status, kErrBadInput);
    return;
  }
  const int32_t *prow = pred + (int64_t)ed2st[src] * n;
  int v = dst;
  for (int steps = 0; v != src; steps++) {
    const int u = prow[v];
    if (u < 0) return;  // unreached: zero gradient
    if (u >= n || steps >= n) {
      atomicOr(status, kErrBadInput);
      return;
    }
    int best = -1;
    float bw = 0.0f;
    for (int e = ro[u]; e < ro[u + 1]; e++)
      if (col[e] == v && (best < 0 || w[e] < bw)) {
        best = e;
        bw = w[e];
      }
    if (best < 0) {
      atomicOr(status, kErrBadInput);
      return;
    }
    atomicAdd(&dw[best], gi);
    v = u;
  }
}

// Dense form: instance b's predecessor matrix P_b (size_b x size_b, leading
// dimension ld_b); the gradient is the dense matrix dW_b (same shape).
struct DenseInst {
  const int32_t *P;
  float *dW;
  int64_t ld;
  int32_t size;
};

__global__ void backward_dense_kernel(const DenseInst *__restrict__ inst, int32_t ninst,
                                      int32_t npairs, const int32_t *__restrict__ b,
                                      const int32_t *__restrict__ s, const int32_t *__restrict__ t,
                                      const float *__restrict__ g, unsigned *status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npairs) return;
  const int bi = b[i];
  if (bi < 0 || bi >= ninst) {
    atomicOr(status, kErrBadInput);
    return;
  }
  const DenseInst I = inst[bi];
  const int src = s[i], dst = t[i];
  if (src < 0 || src >= I.size || dst < 0 || dst >= I.size) {
    atomicOr(status, kErrBadInput);
    return;
  }
  const float gi = g[i];
  const int32_t *prow = I.P + (int64_t)src * I.ld;
  int v = dst;
  for (int steps = 0; v != src; steps++) {
    const int u = prow[v];
    if (u < 0) return;
    if (u >= I.size || steps >= I.size) {
      atomicOr(status, kErrBadInput);
      return;
    }
    atomicAdd(&I.dW[(int64_t)u * I.ld + v], gi);
    v = u;
  }
}

}  // namespace

cudaError_t launch_backward_graph(int32_t n, const int32_t *ro, const int32_t *col, const float *w,
                                  const int32_t *ed2st, const int32_t *pred, int32_t npairs,
                                  const int32_t *s, const int32_t *t, const float *g, float *dw,
                                  unsigned *status, cudaStream_t st) {
  if (npairs <= 0) return cudaSuccess;
  backward_graph_kernel<<<(npairs + 255) / 256, 256, 0, st>>>(n, ro, col, w, ed2st, pred, npairs,
                                                              s, t, g, dw, status);
  return cudaGetLastError();
}

cudaError_t launch_backward_dense(const void *inst, int32_t ninst, int32_t npairs,
                                  const int32_t *b, const int32_t *s, const int32_t *t,
                                  const float *g, unsigned *status, cudaStream_t st) {
  if (npairs <= 0) return cudaSuccess;
  backward_dense_kernel<<<(npairs + 255) / 256, 256, 0, st>>>(
      static_cast<const DenseInst *>(inst), ninst, npairs, b, s, t, g, status);
  return cudaGetLastError();
}

size_t dense_inst_bytes() { return sizeof(DenseInst); }

void fill_dense_inst(void *dst, const int32_t *P, float *dW, int64_t ld, int32_t size) {
  DenseInst *d = static_cast<DenseInst *>(dst);
  d->P = P;
  d->dW = dW;
  d->ld = ld;
  d->size = size;
}

}  // namespace fapk
