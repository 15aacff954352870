// sssp.cu -- batched single-source shortest paths from boundary vertices.
//
// Reference counterparts: handle_boundry_path / batched_sssp_path /
// dijkstra_path (fap/kernel/batch_sssp.h:79-114, 232-303) on the CPU and
// multi_source_Nvidia_sssp[_data_on_gpu] (fap/kernel/cuda/batch_sssp.cu:
// 177-288, 361-414) on the GPU, which runs one source at a time with a host
// round trip per relaxation sweep and computes no predecessors.
//
// Design (GB300): one CTA owns a batch of LANES (16 or 32) sources, one per
// lane of a lane group; a warp relaxes 32 / LANES frontier vertices at once.
// Distances live in a vertex-major scratch table dvm[v][lane], so relaxing an
// edge u->v for the whole batch touches one 64- or 128-byte line.
//
// The search is a near-far delta-stepping (chaotic relaxation with a moving
// threshold): vertices whose improved distance is below the threshold T join
// the next near frontier, the others wait in a far list; when the near
// frontier empties, T grows by delta and the far list is split again.  This
// keeps the re-relaxations of plain Bellman-Ford on long weighted paths (road
// networks) down while every phase stays data-parallel.  Relaxation is an
// atomicMin on the distance bits (non-negative floats, doubles and the int32
// encoding all order like their bits); per-vertex stamps let a vertex enter a
// frontier once per step.  No host round trip: the loop ends when both
// frontiers are empty, or at a step cap that sets an error flag instead of
// spinning.  The result is the fixpoint dist[v] = min_u fl(dist[u] + w(u,v)),
// which for positive weights is unique whatever the order of relaxations, so
// the FP32 distances equal those of the reference's FP32 Dijkstra bit for
// bit.  With ACC64 (FP32 weights) the search runs in FP64 and rounds once at
// the end, which puts the result within an ulp of the FP64 distances.
//
// Predecessors are computed after convergence from the in-edges, with the
// reference Dijkstra's tie rule: Dijkstra settles vertices in (distance, id)
// order and only a strict improvement sets path[v], so path[v] is the
// in-neighbour u with fl(dist[u] + w) == dist[v] that comes first in
// (dist[u], u) order.  Each warp then transposes its own 32-vertex blocks
// through a private shared-memory tile (no CTA barrier) so that every source
// row is written with coalesced stores.

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

constexpr int kSsspThreads = 512;
constexpr int kSsspWarps = kSsspThreads / 32;

// dvm (n x 32 four-byte or n x 16 eight-byte entries) + near/far frontiers
// (2 + 2), n ints each.  The near and far stamps (2n ints per slot) live in
// SsspArgs::stamps, which is zeroed when it is allocated.
__host__ __device__ inline size_t slot_bytes(int32_t n) {
  size_t b = (size_t)n * 32 * 4 + (size_t)n * 4 * 4;
  return (b + 255) & ~(size_t)255;
}

// Per-warp transpose tile of the output pass (32 vertices x LANES sources).
template <int LANES>
struct OutTile {
  unsigned d[32][LANES + 1];
  int32_t p[32][LANES + 1];
};
template <int LANES>
constexpr size_t out_smem() { return sizeof(OutTile<LANES>) * kSsspWarps; }

template <typename T, bool ACC64>
struct Acc;
template <typename T>
struct Acc<T, false> {  // distances kept in the output type
  using V = T;
  using K = unsigned;
  static __device__ __forceinline__ K key(V v) { return Dist<T>::bits(v); }
  static __device__ __forceinline__ V val(K k) { return Dist<T>::from_bits(k); }
  static __device__ __forceinline__ V weight(unsigned wb) { return Dist<T>::from_bits(wb); }
  static __device__ __forceinline__ K inf() { return Dist<T>::bits(Dist<T>::inf()); }
  static __device__ __forceinline__ unsigned out(K k) { return k; }
  static __device__ __forceinline__ V from_double(double x) { return (V)x; }
};
template <>
struct Acc<float, true> {  // FP32 weights, FP64 search
  using V = double;
  using K = unsigned long long;
  static __device__ __forceinline__ K key(V v) { return (K)__double_as_longlong(v); }
  static __device__ __forceinline__ V val(K k) { return __longlong_as_double((long long)k); }
  static __device__ __forceinline__ V weight(unsigned wb) { return (double)__uint_as_float(wb); }
  static __device__ __forceinline__ K inf() { return key((double)Dist<float>::inf()); }
  static __device__ __forceinline__ unsigned out(K k) {
    return k >= inf() ? __float_as_uint(Dist<float>::inf()) : __float_as_uint((float)val(k));
  }
  static __device__ __forceinline__ V from_double(double x) { return x; }
};

template <typename T, bool PRED, int LANES, bool ACC64>
__global__ void __launch_bounds__(kSsspThreads)
    sssp_kernel(SsspArgs a) {
  using A = Acc<T, ACC64>;
  using V = typename A::V;
  using K = typename A::K;
  constexpr int VPW = 32 / LANES;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / LANES, sl = lane % LANES;
  const unsigned group_mask = LANES == 32 ? 0xffffffffu : (0xffffu << (16 * sub));
  const int32_t n = a.n;
  unsigned char *base = static_cast<unsigned char *>(a.scratch) + (size_t)blockIdx.x * slot_bytes(n);
  K *dvm = reinterpret_cast<K *>(base);
  int32_t *nearq[2], *farq[2];
  nearq[0] = reinterpret_cast<int32_t *>(base + (size_t)n * 32 * 4);
  nearq[1] = nearq[0] + n;
  farq[0] = nearq[1] + n;
  farq[1] = farq[0] + n;
  int32_t *stamp = a.stamps + (size_t)blockIdx.x * 2 * n;
  int32_t *fstamp = stamp + n;
  const unsigned *wb = static_cast<const unsigned *>(a.w);
  const unsigned *iwb = static_cast<const unsigned *>(a.iw);
  const K INF = A::inf();
  const V delta = A::from_double(a.delta);

  extern __shared__ __align__(16) unsigned char sssp_smem[];
  OutTile<LANES> &tile = reinterpret_cast<OutTile<LANES> *>(sssp_smem)[warp];
  __shared__ int s_near[2], s_far[2];
  __shared__ K s_minfar;

  // Stamps persist across launches; each slot continues its own epoch count
  // so that no stamp left by an earlier launch can equal a new epoch.
  int epoch = a.slot_epoch[blockIdx.x];
  unsigned local_max = 0;  // largest finite int32 distance this thread wrote
  unsigned long long st_steps = 0, st_splits = 0, st_relaxed = 0, st_scanned = 0, st_batches = 0;
  for (int b = blockIdx.x; b < a.nbatches; b += gridDim.x) {
    int steps = 0;  // BF steps + far splits of this batch (capped)
    const int cnt = a.batches[b].count;
    const int my_src = sl < cnt ? a.batches[b].src[sl] : -1;
    for (size_t i = threadIdx.x; i < (size_t)n * LANES; i += blockDim.x) dvm[i] = INF;
    if (threadIdx.x == 0) {
      s_near[0] = s_near[1] = 0;
      s_far[0] = s_far[1] = 0;
    }
    epoch++;
    int far_epoch = ++epoch;
    __syncthreads();
    if (threadIdx.x < LANES && my_src >= 0 && my_src < n) {
      dvm[(size_t)my_src * LANES + sl] = A::key((V)0);
      if (atomicExch(&stamp[my_src], epoch) != epoch) {
        const int pos = atomicAdd(&s_near[0], 1);
        nearq[0][pos] = my_src;
      }
    } else if (threadIdx.x < LANES && my_src >= n) {
      atomicOr(a.status, kErrBadInput);
    }
    __syncthreads();

    V thr = delta;
    int cur = 0, fcur = 0;
    bool capped = false;
    for (;;) {
      // ---- near phase: BF steps over the near frontier ----
      for (;;) {
        const int f = s_near[cur];
        if (f == 0) break;
        if (++steps > a.iter_cap) {
          capped = true;
          break;
        }
        st_steps++;
        st_relaxed += (unsigned long long)f;
        epoch++;
        const int32_t *F = nearq[cur];
        int32_t *N = nearq[cur ^ 1];
        int32_t *FAR = farq[fcur];
        for (int fb = warp * VPW; fb < f; fb += kSsspWarps * VPW) {
          const int idx = fb + sub;
          const bool has = idx < f;
          const int u = has ? __ldcg(&F[idx]) : 0;
          const K duk = has ? __ldcg(&dvm[(size_t)u * LANES + sl]) : INF;
          const V du = A::val(duk);
          const int e0 = has ? a.ro[u] : 0;
          const int deg = has ? a.ro[u + 1] - e0 : 0;
          int maxdeg = deg;
          if (VPW == 2) maxdeg = max(deg, __shfl_xor_sync(0xffffffffu, deg, 16));
          // Edges in groups of 4: the neighbour ids, weights and current
          // distances of a group are loaded before any atomic, so a vertex
          // costs a few dependent round trips rather than a few per edge.
          constexpr int G = 4;
          for (int e = 0; e < maxdeg; e += G) {
            int v[G];
            K cur_k[G], ck[G];
            V c[G];
            bool live[G];
#pragma unroll
            for (int q = 0; q < G; q++) {
              live[q] = e + q < deg;
              v[q] = live[q] ? a.col[e0 + e + q] : 0;
              c[q] = live[q] ? du + A::weight(wb[e0 + e + q]) : (V)0;
            }
#pragma unroll
            for (int q = 0; q < G; q++) {
              ck[q] = A::key(c[q]);
              cur_k[q] = (live[q] && duk < INF) ? __ldcg(&dvm[(size_t)v[q] * LANES + sl]) : (K)0;
            }
#pragma unroll
            for (int q = 0; q < G; q++) {
              bool imp = false, nearv = false;
              if (live[q] && duk < INF && ck[q] < cur_k[q]) {
                imp = ck[q] < atomicMin(&dvm[(size_t)v[q] * LANES + sl], ck[q]);
                nearv = imp && c[q] < thr;
              }
              const unsigned bi = __ballot_sync(0xffffffffu, imp) & group_mask;
              const unsigned bn = __ballot_sync(0xffffffffu, nearv) & group_mask;
              if (bi != 0u && sl == 0) {
                if (bn != 0u) {
                  if (atomicExch(&stamp[v[q]], epoch) != epoch) N[atomicAdd(&s_near[cur ^ 1], 1)] = v[q];
                } else if (atomicExch(&fstamp[v[q]], far_epoch) != far_epoch) {
                  FAR[atomicAdd(&s_far[fcur], 1)] = v[q];
                }
              }
            }
          }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_near[cur] = 0;
        cur ^= 1;
        __syncthreads();
      }
      if (capped) break;
      const int nf = s_far[fcur];
      if (nf == 0) break;
      // ---- split the far list at the next threshold ----
      if (++steps > a.iter_cap) {
        capped = true;
        break;
      }
      thr += delta;
      st_splits++;
      st_scanned += (unsigned long long)nf;
      epoch++;
      const int new_far_epoch = ++epoch;
      if (threadIdx.x == 0) s_minfar = INF;
      __syncthreads();
      const int32_t *FAR = farq[fcur];
      int32_t *NFAR = farq[fcur ^ 1];
      for (int fb = warp * VPW; fb < nf; fb += kSsspWarps * VPW) {
        const int idx = fb + sub;
        const bool has = idx < nf;
        const int v = has ? __ldcg(&FAR[idx]) : 0;
        K m = has ? __ldcg(&dvm[(size_t)v * LANES + sl]) : INF;
#pragma unroll
        for (int o = LANES / 2; o >= 1; o >>= 1) {
          const K other = __shfl_xor_sync(0xffffffffu, m, o);
          m = other < m ? other : m;
        }
        if (has && sl == 0) {
          if (A::val(m) < thr) {
            if (atomicExch(&stamp[v], epoch) != epoch) nearq[cur][atomicAdd(&s_near[cur], 1)] = v;
          } else if (atomicExch(&fstamp[v], new_far_epoch) != new_far_epoch) {
            NFAR[atomicAdd(&s_far[fcur ^ 1], 1)] = v;
            atomicMin(&s_minfar, m);
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) s_far[fcur] = 0;
      // nothing below the new threshold: jump it to the far minimum
      if (s_near[cur] == 0 && s_minfar < INF) thr = A::val(s_minfar) + delta;
      fcur ^= 1;
      far_epoch = new_far_epoch;
      __syncthreads();
    }
    if (capped) {
      if (threadIdx.x == 0) atomicOr(a.status, kErrSsspCap);
      break;
    }

    // ---- predecessors and transposed output: warps work on their own
    // 32-vertex blocks and synchronize only within the warp ----
    for (int v0 = warp * 32; v0 < n; v0 += kSsspWarps * 32) {
      for (int vi = sub; vi < 32; vi += VPW) {
        const int v = v0 + vi;
        unsigned dv_out = Dist<T>::bits(Dist<T>::inf());
        int32_t p = -1;
        if (v < n && sl < cnt) {
          const K dvk = __ldcg(&dvm[(size_t)v * LANES + sl]);
          dv_out = A::out(dvk);
          if (dvk < INF) {
            if (!std::is_same<T, float>::value) local_max = max(local_max, dv_out);
            if (PRED) {
              if (v == my_src) {
                p = v;
              } else {
                K bdu = ~(K)0;
                int bu = -1;
                const V dv = A::val(dvk);
                for (int e = a.iro[v]; e < a.iro[v + 1]; e++) {
                  const int u = a.icol[e];
                  const K duk = __ldcg(&dvm[(size_t)u * LANES + sl]);
                  if (duk >= INF) continue;
                  if (A::val(duk) + A::weight(iwb[e]) == dv && (duk < bdu || (duk == bdu && u < bu))) {
                    bdu = duk;
                    bu = u;
                  }
                }
                p = bu;
              }
            }
          }
        }
        tile.d[vi][sl] = dv_out;
        tile.p[vi][sl] = p;
      }
      __syncwarp();
      const int col = v0 + lane;
      if (col < n) {
        for (int s = 0; s < cnt; s++) {
          const int64_t off = a.batches[b].row_off[s] + col;
          static_cast<unsigned *>(a.dist)[off] = tile.d[lane][s];
          if (PRED) a.pred[off] = tile.p[lane][s];
        }
      }
      __syncwarp();
    }
    __syncthreads();  // dvm and the frontiers are reset by the next batch
    st_batches++;
  }
  if (threadIdx.x == 0) {
    a.slot_epoch[blockIdx.x] = epoch;
    if (a.stats != nullptr) {
      atomicAdd(&a.stats[0], st_steps);
      atomicAdd(&a.stats[1], st_splits);
      atomicAdd(&a.stats[2], st_relaxed);
      atomicAdd(&a.stats[3], st_scanned);
      atomicAdd(&a.stats[4], st_batches);
    }
  }
  if (a.maxd != nullptr) {
    local_max = __reduce_max_sync(0xffffffffu, local_max);
    if (lane == 0 && local_max) atomicMax(a.maxd, local_max);
  }
}

template <typename T, bool PRED, int LANES, bool ACC64>
cudaError_t launch_one(const SsspArgs &a, cudaStream_t st) {
  sssp_kernel<T, PRED, LANES, ACC64><<<a.slots, kSsspThreads, out_smem<LANES>(), st>>>(a);
  return cudaGetLastError();
}

template <typename T, bool PRED>
cudaError_t launch_t(const SsspArgs &a, cudaStream_t st) {
  if (a.acc64) {
    if constexpr (std::is_same<T, float>::value) return launch_one<float, PRED, 16, true>(a, st);
    return cudaErrorInvalidValue;
  }
  if (a.lanes == 16) return launch_one<T, PRED, 16, false>(a, st);
  return launch_one<T, PRED, 32, false>(a, st);
}

template <typename T, bool PRED, int LANES, bool ACC64>
cudaError_t set_attr() {
  return cudaFuncSetAttribute(sssp_kernel<T, PRED, LANES, ACC64>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)out_smem<LANES>());
}

}  // namespace

size_t sssp_slot_bytes(int32_t n) { return slot_bytes(n); }
int sssp_threads() { return kSsspThreads; }

cudaError_t init_sssp_kernels() {
  cudaError_t e;
#define FAP_SSSP_ATTR(T, P, L, A) \
  if ((e = set_attr<T, P, L, A>()) != cudaSuccess) return e;
  FAP_SSSP_ATTR(float, true, 16, false)
  FAP_SSSP_ATTR(float, true, 32, false)
  FAP_SSSP_ATTR(float, false, 16, false)
  FAP_SSSP_ATTR(float, false, 32, false)
  FAP_SSSP_ATTR(uint32_t, true, 16, false)
  FAP_SSSP_ATTR(uint32_t, true, 32, false)
  FAP_SSSP_ATTR(uint32_t, false, 16, false)
  FAP_SSSP_ATTR(uint32_t, false, 32, false)
  FAP_SSSP_ATTR(float, true, 16, true)
  FAP_SSSP_ATTR(float, false, 16, true)
#undef FAP_SSSP_ATTR
  return cudaSuccess;
}

cudaError_t launch_sssp(bool f32, const SsspArgs &a, cudaStream_t st) {
  if (a.nbatches <= 0 || a.slots <= 0) return cudaSuccess;
  if (a.lanes != 16 && a.lanes != 32) return cudaErrorInvalidValue;
  if (a.acc64 && (!f32 || a.lanes != 16)) return cudaErrorInvalidValue;
  if (!(a.delta > 0.0)) return cudaErrorInvalidValue;
  const bool pred = a.pred != nullptr;
  if (f32) return pred ? launch_t<float, true>(a, st) : launch_t<float, false>(a, st);
  return pred ? launch_t<uint32_t, true>(a, st) : launch_t<uint32_t, false>(a, st);
}

int sssp_lanes_for(int64_t sources_total, int64_t batches32, int sm_count) {
  // Half-warp batches double the CTA count and the frontier vertices a warp
  // relaxes at once; worth it while 32-source batches leave SMs idle.
  (void)sources_total;
  return batches32 < 2LL * sm_count ? 16 : 32;
}

}  // namespace fapk
