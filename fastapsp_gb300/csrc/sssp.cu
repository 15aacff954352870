// sssp.cu -- batched single-source shortest paths from boundary vertices.
//
// Reference counterparts: handle_boundry_path / batched_sssp_path /
// dijkstra_path (fap/kernel/batch_sssp.h:79-114, 232-303) on the CPU and
// multi_source_Nvidia_sssp[_data_on_gpu] (fap/kernel/cuda/batch_sssp.cu:
// 177-288, 361-414) on the GPU, which runs one source at a time with a host
// round trip per relaxation sweep and computes no predecessors.
//
// Design (GB300): one CTA owns a batch of up to 32 sources, one per warp lane.
// Its distances live in a vertex-major scratch array dvm[v][lane], so a warp
// relaxing an edge u->v for all 32 sources touches one 128-byte line.  The CTA
// runs a frontier Bellman-Ford (chaotic relaxation): every warp takes frontier
// vertices, relaxes their out-edges for all lanes with atomicMin (unsigned
// order = distance order for non-negative floats and for the int32 encoding),
// and appends improved vertices to the next frontier once (per-vertex stamps).
// No host round trip: the loop ends when the frontier is empty, or at an
// iteration cap, which sets an error flag instead of spinning.  A vertex is
// finished when no relaxation lowers it further, i.e. at the fixpoint
// dist[v] = min_u fl(dist[u] + w(u,v)); for positive weights that fixpoint is
// unique, so the distances equal those of the reference's FP32 Dijkstra bit
// for bit.
//
// Predecessors are computed after convergence from the in-edges, with the
// reference Dijkstra's tie rule: Dijkstra settles vertices in (distance, id)
// order and only a strict improvement sets path[v], so path[v] is the
// in-neighbour u with fl(dist[u] + w) == dist[v] that comes first in
// (dist[u], u) order.  The CTA then transposes 32x32 tiles through shared
// memory so that each source's output row is written with coalesced stores.

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

constexpr int kSsspThreads = 512;

__host__ __device__ inline size_t slot_bytes(int32_t n) {
  size_t b = (size_t)n * 32 * 4 + (size_t)n * 2 * 4;
  return (b + 255) & ~(size_t)255;
}

// LANES sources per batch (16 or 32): a warp relaxes 32 / LANES frontier
// vertices at once, each for LANES sources.
template <typename T, bool PRED, int LANES>
__global__ void __launch_bounds__(kSsspThreads)
    sssp_lanes_kernel(SsspArgs a) {
  constexpr int VPW = 32 / LANES;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / LANES, sl = lane % LANES;
  const unsigned group_mask = LANES == 32 ? 0xffffffffu : (0xffffu << (16 * sub));
  const int nwarps = blockDim.x >> 5;
  const int32_t n = a.n;
  unsigned char *base = static_cast<unsigned char *>(a.scratch) + (size_t)blockIdx.x * slot_bytes(n);
  unsigned *dvm = reinterpret_cast<unsigned *>(base);
  int32_t *fr[2];
  fr[0] = reinterpret_cast<int32_t *>(dvm + (size_t)n * 32);
  fr[1] = fr[0] + n;
  int32_t *stamp = a.stamps + (size_t)blockIdx.x * n;
  const unsigned *wb = static_cast<const unsigned *>(a.w);
  const unsigned *iwb = static_cast<const unsigned *>(a.iw);
  const unsigned INF = Dist<T>::bits(Dist<T>::inf());

  __shared__ int s_count[2];
  __shared__ unsigned tile_d[32][33];
  __shared__ int32_t tile_p[32][33];

  // Stamps persist across launches; each slot continues its own epoch count
  // so that no stamp left by an earlier launch can equal a new epoch.
  int epoch = a.slot_epoch[blockIdx.x];
  unsigned local_max = 0;  // largest finite distance this thread wrote
  for (int b = blockIdx.x; b < a.nbatches; b += gridDim.x) {
    const int cnt = a.batches[b].count;
    const int my_src = sl < cnt ? a.batches[b].src[sl] : -1;
    for (size_t i = threadIdx.x; i < (size_t)n * LANES; i += blockDim.x) dvm[i] = INF;
    if (threadIdx.x == 0) {
      s_count[0] = 0;
      s_count[1] = 0;
    }
    epoch++;
    __syncthreads();
    if (threadIdx.x < LANES && my_src >= 0 && my_src < n) {
      dvm[(size_t)my_src * LANES + sl] = 0u;
      if (atomicExch(&stamp[my_src], epoch) != epoch) {
        int pos = atomicAdd(&s_count[0], 1);
        fr[0][pos] = my_src;
      }
    } else if (threadIdx.x < LANES && my_src >= n) {
      atomicOr(a.status, kErrBadInput);
    }
    __syncthreads();

    int cur = 0, it = 0;
    for (;;) {
      const int f = s_count[cur];
      if (f == 0) break;
      if (it >= a.iter_cap) {
        if (threadIdx.x == 0) atomicOr(a.status, kErrSsspCap);
        break;
      }
      it++;
      epoch++;
      const int32_t *F = fr[cur];
      int32_t *N = fr[cur ^ 1];
      for (int fb = warp * VPW; fb < f; fb += nwarps * VPW) {
        const int idx = fb + sub;
        const bool has = idx < f;
        const int u = has ? __ldcg(&F[idx]) : 0;
        const unsigned du = has ? __ldcg(&dvm[(size_t)u * LANES + sl]) : INF;
        const int e0 = has ? a.ro[u] : 0;
        const int deg = has ? a.ro[u + 1] - e0 : 0;
        int maxdeg = deg;
        if (VPW == 2) maxdeg = max(deg, __shfl_xor_sync(0xffffffffu, deg, 16));
        for (int e = 0; e < maxdeg; e++) {
          bool imp = false;
          int v = 0;
          if (e < deg) {
            v = a.col[e0 + e];
            if (du < INF) {
              const unsigned cand =
                  Dist<T>::bits(Dist<T>::add(Dist<T>::from_bits(du), Dist<T>::from_bits(wb[e0 + e])));
              unsigned *p = &dvm[(size_t)v * LANES + sl];
              if (cand < __ldcg(p)) imp = cand < atomicMin(p, cand);
            }
          }
          const unsigned bal = __ballot_sync(0xffffffffu, imp) & group_mask;
          if (bal != 0u && sl == 0) {
            if (atomicExch(&stamp[v], epoch) != epoch) {
              const int pos = atomicAdd(&s_count[cur ^ 1], 1);
              N[pos] = v;
            }
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) s_count[cur] = 0;
      cur ^= 1;
      __syncthreads();
    }

    // Predecessors and transposed output, 32 vertices at a time.
    for (int v0 = 0; v0 < n; v0 += 32) {
      for (int vi = warp * VPW + sub; vi < 32; vi += nwarps * VPW) {
        const int v = v0 + vi;
        unsigned dv = INF;
        int32_t p = -1;
        if (v < n) {
          dv = __ldcg(&dvm[(size_t)v * LANES + sl]);
          if (PRED && sl < cnt && dv < INF) {
            if (v == my_src) {
              p = v;
            } else {
              unsigned bdu = 0xffffffffu;
              int bu = -1;
              for (int e = a.iro[v]; e < a.iro[v + 1]; e++) {
                const int u = a.icol[e];
                const unsigned du = __ldcg(&dvm[(size_t)u * LANES + sl]);
                if (du >= INF) continue;
                const unsigned s =
                    Dist<T>::bits(Dist<T>::add(Dist<T>::from_bits(du), Dist<T>::from_bits(iwb[e])));
                if (s == dv && (du < bdu || (du == bdu && u < bu))) {
                  bdu = du;
                  bu = u;
                }
              }
              p = bu;
            }
          }
        }
        if (sl < cnt && dv < INF) local_max = max(local_max, dv);
        tile_d[vi][sl] = dv;
        tile_p[vi][sl] = p;
      }
      __syncthreads();
      const int col = v0 + lane;
      for (int s = warp; s < cnt; s += nwarps) {
        if (col < n) {
          const int64_t off = a.batches[b].row_off[s] + col;
          static_cast<unsigned *>(a.dist)[off] = tile_d[lane][s];
          if (PRED) a.pred[off] = tile_p[lane][s];
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) a.slot_epoch[blockIdx.x] = epoch;
  if (a.maxd != nullptr) {
    local_max = __reduce_max_sync(0xffffffffu, local_max);
    if (lane == 0 && local_max) atomicMax(a.maxd, local_max);
  }
}

template <typename T, bool PRED>
void launch_t(const SsspArgs &a, cudaStream_t st) {
  if (a.lanes == 16) sssp_lanes_kernel<T, PRED, 16><<<a.slots, kSsspThreads, 0, st>>>(a);
  else sssp_lanes_kernel<T, PRED, 32><<<a.slots, kSsspThreads, 0, st>>>(a);
}

}  // namespace

size_t sssp_slot_bytes(int32_t n) { return slot_bytes(n); }
int sssp_threads() { return kSsspThreads; }

cudaError_t launch_sssp(bool f32, const SsspArgs &a, cudaStream_t st) {
  if (a.nbatches <= 0 || a.slots <= 0) return cudaSuccess;
  if (a.lanes != 16 && a.lanes != 32) return cudaErrorInvalidValue;
  const bool pred = a.pred != nullptr;
  if (f32) {
    if (pred) launch_t<float, true>(a, st); else launch_t<float, false>(a, st);
  } else {
    if (pred) launch_t<uint32_t, true>(a, st); else launch_t<uint32_t, false>(a, st);
  }
  return cudaGetLastError();
}

int sssp_lanes_for(int64_t sources_total, int64_t batches32, int sm_count) {
  // Half-warp batches double the CTA count and the frontier vertices a warp
  // relaxes at once; worth it while 32-source batches leave SMs idle.
  (void)sources_total;
  return batches32 < 2LL * sm_count ? 16 : 32;
}

}  // namespace fapk
