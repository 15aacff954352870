// sssp.cu -- batched single-source shortest paths from boundary vertices.
//
// Reference counterparts: handle_boundry_path / batched_sssp_path /
// dijkstra_path (fap/kernel/batch_sssp.h:79-114, 232-303) on the CPU and
// multi_source_Nvidia_sssp[_data_on_gpu] (fap/kernel/cuda/batch_sssp.cu:
// 177-288, 361-414) on the GPU, which runs one source at a time with a host
// round trip per relaxation sweep and computes no predecessors.
//
// Design (GB300): one CTA owns a batch of LANES (8, 16 or 32) sources, one per
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
// encoding all order like their bits); frontier bitmaps let a vertex enter a
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

#include <algorithm>
#include <type_traits>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

constexpr int kSsspThreads = 512;
constexpr int kSsspWarps = kSsspThreads / 32;
constexpr int kOutThreads = 256;  // the separate output kernel

// dvm (n x 32 four-byte or n x 16 eight-byte entries; wide: n x 32
// eight-byte entries) + near/far frontiers (2 + 2), n ints each.
__host__ __device__ inline size_t dvm_bytes(int32_t n, bool wide) { return (size_t)n * (wide ? 256 : 128); }
__host__ __device__ inline size_t slot_bytes(int32_t n, bool wide = false) {
  size_t b = dvm_bytes(n, wide) + (size_t)n * 4 * 4;
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

// FP32 graphs whose tables hold exact 64-bit fixed-point distances (the
// boundary-graph method, bgraph.cu): integer comparisons against the in-edge
// weights in the same units, one rounding to FP32 at the end.
struct AccFix {
  using V = unsigned long long;
  using K = unsigned long long;
  static __device__ __forceinline__ V val(K k) { return k; }
  static __device__ __forceinline__ K inf() { return ~0ull; }  // the real bound is SsspArgs::fix_inf
};

// Predecessors and transposed output of one 32-vertex block of batch b (the
// calling warp's; the warp synchronizes only with itself).  A lane group
// takes two vertices at a time and scans their in-edge lists side by side
// (edge j of both per iteration), so their loads overlap; the block then
// goes through the warp's shared-memory tile so that every source row is
// written with coalesced stores.
template <typename T, bool PRED, int LANES, bool ACC64, bool FIX = false>
__device__ __forceinline__ void sssp_out_block(
    const SsspArgs &a, const typename std::conditional<FIX, AccFix, Acc<T, ACC64>>::type::K *dvm, int b,
    int cnt, int my_src, int v0, OutTile<LANES> &tile, unsigned &local_max) {
  using A = typename std::conditional<FIX, AccFix, Acc<T, ACC64>>::type;
  using V = typename A::V;
  using K = typename A::K;
  using W = typename std::conditional<FIX, unsigned long long, unsigned>::type;
  constexpr int VPW = 32 / LANES;
  const int lane = threadIdx.x & 31;
  const int sub = lane / LANES, sl = lane % LANES;
  const int32_t n = a.n;
  const unsigned *iwb = static_cast<const unsigned *>(a.iw);
  const K INF = FIX ? (K)a.fix_inf : A::inf();
  for (int vb = 0; vb < 32; vb += 2 * VPW) {
    int vv[2], e0[2], deg[2], bu[2];
    K dk[2], bdu[2];
    V dvv[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
      vv[i] = v0 + vb + i * VPW + sub;
      const bool in = vv[i] < n;
      dk[i] = (in && sl < cnt) ? __ldcg(&dvm[(size_t)vv[i] * LANES + sl]) : INF;
      dvv[i] = A::val(dk[i]);
      e0[i] = (PRED && in) ? a.iro[vv[i]] : 0;
      deg[i] = (PRED && in) ? a.iro[vv[i] + 1] - e0[i] : 0;
      bdu[i] = ~(K)0;
      bu[i] = -1;
    }
    if (PRED) {
      int dmax = max(deg[0], deg[1]);
#pragma unroll
      for (int o = LANES; o < 32; o <<= 1) dmax = max(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
      // vertices that no source of the batch reached need no scan
      if (!__any_sync(0xffffffffu, dk[0] < INF || dk[1] < INF)) dmax = 0;
      for (int j = 0; j < dmax; j++) {
        int u[2];
        W wq[2];
        K duk[2];
#pragma unroll
        for (int i = 0; i < 2; i++) {
          const bool has = j < deg[i];
          u[i] = has ? a.icol[e0[i] + j] : 0;
          if constexpr (FIX)
            wq[i] = has ? a.iwfix[e0[i] + j] : 0ull;
          else
            wq[i] = has ? iwb[e0[i] + j] : 0u;
          duk[i] = (has && dk[i] < INF) ? __ldcg(&dvm[(size_t)u[i] * LANES + sl]) : INF;
        }
#pragma unroll
        for (int i = 0; i < 2; i++) {
          bool tight;
          if constexpr (FIX)
            tight = duk[i] + wq[i] == dvv[i];
          else
            tight = A::val(duk[i]) + A::weight(wq[i]) == dvv[i];
          const bool better = duk[i] < INF && tight &&
                              (duk[i] < bdu[i] || (duk[i] == bdu[i] && u[i] < bu[i]));
          bdu[i] = better ? duk[i] : bdu[i];
          bu[i] = better ? u[i] : bu[i];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
      unsigned dv_out = Dist<T>::bits(Dist<T>::inf());
      int32_t p = -1;
      if (dk[i] < INF) {
        if constexpr (FIX)
          dv_out = __float_as_uint((float)((double)dk[i] * a.fix_scale));  // exact product, one rounding
        else
          dv_out = A::out(dk[i]);
        if (!std::is_same<T, float>::value) local_max = max(local_max, dv_out);
        if (PRED) p = vv[i] == my_src ? vv[i] : bu[i];
      }
      tile.d[vb + i * VPW + sub][sl] = dv_out;
      tile.p[vb + i * VPW + sub][sl] = p;
    }
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

// Output pass of every batch at once, after a search launch that deferred it
// (one batch per search CTA, so batch b's distance table is slot b): block
// (x, b) has its warps take 32-vertex blocks x * warps + w of batch b.
template <typename T, bool PRED, int LANES, bool ACC64, bool FIX = false>
__global__ void __launch_bounds__(kOutThreads)
    sssp_output_kernel(SsspArgs a) {
  using A = typename std::conditional<FIX, AccFix, Acc<T, ACC64>>::type;
  using K = typename A::K;
  extern __shared__ __align__(16) unsigned char out_smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  OutTile<LANES> &tile = reinterpret_cast<OutTile<LANES> *>(out_smem_raw)[warp];
  const int b = blockIdx.y;
  const K *dvm = reinterpret_cast<const K *>(static_cast<const unsigned char *>(a.scratch) +
                                             (size_t)b * slot_bytes(a.n, (ACC64 || FIX) && LANES == 32));
  const int cnt = a.batches[b].count;
  const int sl = lane % LANES;
  const int my_src = sl < cnt ? a.batches[b].src[sl] : -1;
  unsigned local_max = 0;
  const int v0 = (blockIdx.x * (kOutThreads / 32) + warp) * 32;
  if (v0 < a.n) sssp_out_block<T, PRED, LANES, ACC64, FIX>(a, dvm, b, cnt, my_src, v0, tile, local_max);
  if (a.maxd != nullptr) {
    local_max = __reduce_max_sync(0xffffffffu, local_max);
    if (lane == 0 && local_max) atomicMax(a.maxd, local_max);
  }
}

// Frontier membership bitmaps: near[2] (entry of the next near frontier,
// alternating per step) and far (entry of the far list), ceil(n / 32) words
// each.  They live in the dynamic shared memory (overlaid on the output
// tiles, which are only used after the search) when they fit there, else in
// the slot's part of SsspArgs::bits.
__host__ __device__ inline size_t bitmap_bytes(int32_t n) { return (size_t)3 * ((n + 31) / 32) * 4; }
constexpr size_t kBitmapSmemMax = 160 * 1024;

__device__ __forceinline__ bool set_bit(unsigned *bits, int v) {
  const unsigned m = 1u << (v & 31);
  return (atomicOr(&bits[v >> 5], m) & m) == 0u;
}
__device__ __forceinline__ void clear_bit(unsigned *bits, int v) {
  atomicAnd(&bits[v >> 5], ~(1u << (v & 31)));
}

// The FP64 search at two CTAs per SM (64 registers, a few spills): on the
// 114,599-vertex road-like graph with 128 parts its 220 batches then run in
// one wave (search 225 -> 179 ms).
template <typename T, bool PRED, int LANES, bool ACC64>
__global__ void __launch_bounds__(kSsspThreads, ACC64 ? 2 : 1)
    sssp_kernel(SsspArgs a) {
  using A = Acc<T, ACC64>;
  using V = typename A::V;
  using K = typename A::K;
  constexpr int VPW = 32 / LANES;  // lane groups (frontier vertices) per warp
  constexpr int R = 2;             // frontier vertices per lane group per sweep
  constexpr int G = 8;             // edges per lane group in flight (<= LANES)
  static_assert(G <= LANES, "lane q of a group files edge target q: every edge in flight needs a lane");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / LANES, sl = lane % LANES;
  const unsigned group_mask = LANES == 32 ? 0xffffffffu : (((1u << LANES) - 1u) << (LANES * sub));
  const int32_t n = a.n;
  constexpr bool kWide = ACC64 && LANES == 32;
  unsigned char *base = static_cast<unsigned char *>(a.scratch) + (size_t)blockIdx.x * slot_bytes(n, kWide);
  K *dvm = reinterpret_cast<K *>(base);
  // near frontiers at nearq0 + {0, n}, far lists at farq0 + {0, n}
  int32_t *const nearq0 = reinterpret_cast<int32_t *>(base + dvm_bytes(n, kWide));
  int32_t *const farq0 = nearq0 + 2 * (size_t)n;
  const unsigned *wb = static_cast<const unsigned *>(a.w);
  const K INF = A::inf();
  const V delta = A::from_double(a.delta);

  extern __shared__ __align__(16) unsigned char sssp_smem[];
  OutTile<LANES> &tile = reinterpret_cast<OutTile<LANES> *>(sssp_smem)[warp];
  const int words = (n + 31) / 32;
  unsigned *bits = bitmap_bytes(n) <= kBitmapSmemMax
                       ? reinterpret_cast<unsigned *>(sssp_smem)
                       : reinterpret_cast<unsigned *>(a.bits) + (size_t)blockIdx.x * 3 * words;
  unsigned *const farbits = bits + 2 * words;  // near bitmaps at bits + {0, words}
  __shared__ int s_near[2], s_far[2];
  __shared__ K s_minfar;

  unsigned local_max = 0;  // largest finite int32 distance this thread wrote
  unsigned long long st_steps = 0, st_splits = 0, st_relaxed = 0, st_scanned = 0, st_batches = 0;
  for (int b = blockIdx.x; b < a.nbatches; b += gridDim.x) {
    int steps = 0;  // BF steps + far splits of this batch (capped)
    const int cnt = a.batches[b].count;
    const int my_src = sl < cnt ? a.batches[b].src[sl] : -1;
    for (size_t i = threadIdx.x; i < (size_t)n * LANES; i += blockDim.x) dvm[i] = INF;
    for (int i = threadIdx.x; i < 3 * words; i += blockDim.x) bits[i] = 0u;
    if (threadIdx.x == 0) {
      s_near[0] = s_near[1] = 0;
      s_far[0] = s_far[1] = 0;
    }
    __syncthreads();
    if (threadIdx.x < LANES && my_src >= 0 && my_src < n) {
      dvm[(size_t)my_src * LANES + sl] = A::key((V)0);
      if (set_bit(bits, my_src)) nearq0[atomicAdd(&s_near[0], 1)] = my_src;
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
        const int32_t *F = nearq0 + (size_t)cur * n;
        int32_t *N = nearq0 + (size_t)(cur ^ 1) * n;
        int32_t *FAR = farq0 + (size_t)fcur * n;
        unsigned *fbits = bits + cur * words, *nbits = bits + (cur ^ 1) * words;
        // A lane group takes R frontier vertices per sweep and walks their
        // concatenated out-edge lists G edges at a time: the loads of a
        // sweep's vertices, of G edges and the G atomics are each issued
        // together, so a sweep costs four dependent round trips.  Two
        // vertices of one group can push the same target: the bitmap keeps
        // one copy.
        for (int fb = warp * VPW * R; fb < f; fb += kSsspWarps * VPW * R) {
          int u[R];
#pragma unroll
          for (int i = 0; i < R; i++) {
            const int idx = fb + i * VPW + sub;
            u[i] = idx < f ? __ldcg(&F[idx]) : -1;
          }
          V du[R];
          bool ok[R];
          int eb[R], pre[R + 1];
          pre[0] = 0;
#pragma unroll
          for (int i = 0; i < R; i++) {
            K k = INF;
            int e0 = 0, deg = 0;
            if (u[i] >= 0) {
              k = __ldcg(&dvm[(size_t)u[i] * LANES + sl]);
              e0 = a.ro[u[i]];
              deg = a.ro[u[i] + 1] - e0;
              if (sl == 0) clear_bit(fbits, u[i]);
            }
            du[i] = A::val(k);
            ok[i] = k < INF;
            pre[i + 1] = pre[i] + deg;
            eb[i] = e0 - pre[i];
          }
          const int tot = pre[R];
          int tmax = tot;  // the longest edge walk of the warp's lane groups
#pragma unroll
          for (int o = LANES; o < 32; o <<= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
          for (int t0 = 0; t0 < tmax; t0 += G) {
            int v[G];
            V c[G];
            bool live[G];
#pragma unroll
            for (int q = 0; q < G; q++) {
              const int t = t0 + q;
              V d = du[0];
              int e = eb[0] + t;
              bool o = ok[0];
#pragma unroll
              for (int i = 1; i < R; i++)
                if (t >= pre[i]) {
                  d = du[i];
                  e = eb[i] + t;
                  o = ok[i];
                }
              const bool in = t < tot;
              v[q] = in ? a.col[e] : 0;
              live[q] = in && o;
              c[q] = live[q] ? d + A::weight(wb[e]) : (V)0;
            }
            K old[G];
#pragma unroll
            for (int q = 0; q < G; q++)
              old[q] = live[q] ? atomicMin(&dvm[(size_t)v[q] * LANES + sl], A::key(c[q])) : (K)0;
            // Which edge targets improved (for any source of the group) and
            // whether below the threshold; then lane q of the group files
            // target q, so the G pushes run side by side.
            unsigned bi[G], bn[G];
#pragma unroll
            for (int q = 0; q < G; q++) {
              const bool imp = live[q] && A::key(c[q]) < old[q];
              bi[q] = __ballot_sync(0xffffffffu, imp) & group_mask;
              bn[q] = __ballot_sync(0xffffffffu, imp && c[q] < thr) & group_mask;
            }
            int mv = v[0];
            unsigned mi = bi[0], mn = bn[0];
#pragma unroll
            for (int q = 1; q < G; q++)
              if (sl == q) {
                mv = v[q];
                mi = bi[q];
                mn = bn[q];
              }
            if (sl < G && mi != 0u) {
              if (mn != 0u) {
                if (set_bit(nbits, mv)) N[atomicAdd(&s_near[cur ^ 1], 1)] = mv;
              } else if (set_bit(farbits, mv)) {
                FAR[atomicAdd(&s_far[fcur], 1)] = mv;
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
      if (threadIdx.x == 0) s_minfar = INF;
      __syncthreads();
      const int32_t *FAR = farq0 + (size_t)fcur * n;
      int32_t *NFAR = farq0 + (size_t)(fcur ^ 1) * n;
      int32_t *NEAR = nearq0 + (size_t)cur * n;
      unsigned *nearbits = bits + cur * words;
      for (int fb = warp * VPW * R; fb < nf; fb += kSsspWarps * VPW * R) {
        int v[R];
        K m[R];
#pragma unroll
        for (int i = 0; i < R; i++) {
          const int idx = fb + i * VPW + sub;
          v[i] = idx < nf ? __ldcg(&FAR[idx]) : -1;
        }
#pragma unroll
        for (int i = 0; i < R; i++) m[i] = v[i] >= 0 ? __ldcg(&dvm[(size_t)v[i] * LANES + sl]) : INF;
#pragma unroll
        for (int i = 0; i < R; i++) {
#pragma unroll
          for (int o = LANES / 2; o >= 1; o >>= 1) {
            const K other = __shfl_xor_sync(0xffffffffu, m[i], o);
            m[i] = other < m[i] ? other : m[i];
          }
          if (v[i] >= 0 && sl == 0) {
            if (A::val(m[i]) < thr) {
              // leaves the far list (its bit is cleared) for the near frontier
              clear_bit(farbits, v[i]);
              if (set_bit(nearbits, v[i])) NEAR[atomicAdd(&s_near[cur], 1)] = v[i];
            } else {
              NFAR[atomicAdd(&s_far[fcur ^ 1], 1)] = v[i];  // stays, bit kept
              atomicMin(&s_minfar, m[i]);
            }
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) s_far[fcur] = 0;
      // nothing below the new threshold: jump it to the far minimum
      if (s_near[cur] == 0 && s_minfar < INF) thr = A::val(s_minfar) + delta;
      fcur ^= 1;
      __syncthreads();
    }
    if (capped) {
      if (threadIdx.x == 0) atomicOr(a.status, kErrSsspCap);
      break;
    }

    // ---- predecessors and transposed output: warps work on their own
    // 32-vertex blocks and synchronize only within the warp.  A lane group
    // takes two vertices at a time and scans their in-edge lists side by
    // side (edge j of both per iteration), so their loads overlap. ----
    if (!a.defer_output)
      for (int v0 = warp * 32; v0 < n; v0 += kSsspWarps * 32)
        sssp_out_block<T, PRED, LANES, ACC64>(a, dvm, b, cnt, my_src, v0, tile, local_max);
    __syncthreads();  // dvm, the frontiers and the bitmaps are reset by the next batch
    st_batches++;
  }
  if (threadIdx.x == 0 && a.stats != nullptr) {
    atomicAdd(&a.stats[0], st_steps);
    atomicAdd(&a.stats[1], st_splits);
    atomicAdd(&a.stats[2], st_relaxed);
    atomicAdd(&a.stats[3], st_scanned);
    atomicAdd(&a.stats[4], st_batches);
  }
  if (a.maxd != nullptr) {
    local_max = __reduce_max_sync(0xffffffffu, local_max);
    if (lane == 0 && local_max) atomicMax(a.maxd, local_max);
  }
}

template <int LANES>
constexpr size_t out_kernel_smem() { return sizeof(OutTile<LANES>) * (kOutThreads / 32); }

// When every batch has its own CTA (and so its own distance table), the
// output pass -- predecessors, transposes and row writes, bound by memory
// latency per vertex -- runs as a second launch over all batches and vertex
// blocks at once instead of inside each batch's CTA.
template <typename T, bool PRED, int LANES, bool ACC64>
cudaError_t launch_one(const SsspArgs &a0, cudaStream_t st) {
  SsspArgs a = a0;
  a.defer_output = a.nbatches <= a.slots ? 1 : 0;
  size_t smem = out_smem<LANES>();
  if (bitmap_bytes(a.n) <= kBitmapSmemMax) smem = std::max(smem, bitmap_bytes(a.n));
  ++launch_count();
  sssp_kernel<T, PRED, LANES, ACC64><<<a.slots, kSsspThreads, smem, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !a.defer_output) return e;
  const dim3 grid((unsigned)((a.n + kOutThreads - 1) / kOutThreads), (unsigned)a.nbatches);
  ++launch_count();
  sssp_output_kernel<T, PRED, LANES, ACC64><<<grid, kOutThreads, out_kernel_smem<LANES>(), st>>>(a);
  return cudaGetLastError();
}

template <typename T, bool PRED, int LANES, bool ACC64, bool FIX = false>
cudaError_t launch_output(const SsspArgs &a, cudaStream_t st) {
  const dim3 grid((unsigned)((a.n + kOutThreads - 1) / kOutThreads), (unsigned)a.nbatches);
  ++launch_count();
  sssp_output_kernel<T, PRED, LANES, ACC64, FIX><<<grid, kOutThreads, out_kernel_smem<LANES>(), st>>>(a);
  return cudaGetLastError();
}

template <typename T, bool PRED>
cudaError_t launch_output_t(const SsspArgs &a, cudaStream_t st) {
  if (a.fix) {
    if constexpr (std::is_same<T, float>::value)
      return a.lanes == 16 ? launch_output<float, PRED, 16, false, true>(a, st)
                           : launch_output<float, PRED, 32, false, true>(a, st);
    return cudaErrorInvalidValue;
  }
  if (a.acc64) {
    if constexpr (std::is_same<T, float>::value)
      return a.lanes == 16 ? launch_output<float, PRED, 16, true>(a, st) : launch_output<float, PRED, 32, true>(a, st);
    return cudaErrorInvalidValue;
  }
  if (a.lanes == 8) return launch_output<T, PRED, 8, false>(a, st);
  if (a.lanes == 16) return launch_output<T, PRED, 16, false>(a, st);
  return launch_output<T, PRED, 32, false>(a, st);
}

template <typename T, bool PRED>
cudaError_t launch_t(const SsspArgs &a, cudaStream_t st) {
  if (a.acc64) {
    if constexpr (std::is_same<T, float>::value)
      return a.lanes == 16 ? launch_one<float, PRED, 16, true>(a, st) : launch_one<float, PRED, 32, true>(a, st);
    return cudaErrorInvalidValue;
  }
  if (a.lanes == 8) return launch_one<T, PRED, 8, false>(a, st);
  if (a.lanes == 16) return launch_one<T, PRED, 16, false>(a, st);
  return launch_one<T, PRED, 32, false>(a, st);
}

template <typename T, bool PRED, int LANES, bool ACC64>
cudaError_t set_attr() {
  cudaError_t e = cudaFuncSetAttribute(sssp_kernel<T, PRED, LANES, ACC64>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)std::max(out_smem<LANES>(), kBitmapSmemMax));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(sssp_output_kernel<T, PRED, LANES, ACC64>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)out_kernel_smem<LANES>());
}

}  // namespace

size_t sssp_slot_bytes(int32_t n, bool wide) { return slot_bytes(n, wide); }
size_t sssp_bits_bytes(int32_t n) { return bitmap_bytes(n) <= kBitmapSmemMax ? 0 : bitmap_bytes(n); }
int sssp_threads() { return kSsspThreads; }

cudaError_t init_sssp_kernels() {
  cudaError_t e;
#define FAP_SSSP_ATTR(T, P, L, A) \
  if ((e = set_attr<T, P, L, A>()) != cudaSuccess) return e;
  FAP_SSSP_ATTR(float, true, 8, false)
  FAP_SSSP_ATTR(float, false, 8, false)
  FAP_SSSP_ATTR(uint32_t, true, 8, false)
  FAP_SSSP_ATTR(uint32_t, false, 8, false)
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
  FAP_SSSP_ATTR(float, true, 32, true)
  FAP_SSSP_ATTR(float, false, 32, true)
#undef FAP_SSSP_ATTR
#define FAP_OUT_FIX_ATTR(P, L)                                                                     \
  if ((e = cudaFuncSetAttribute(sssp_output_kernel<float, P, L, false, true>,                      \
                                cudaFuncAttributeMaxDynamicSharedMemorySize,                       \
                                (int)out_kernel_smem<L>())) != cudaSuccess)                        \
    return e;
  FAP_OUT_FIX_ATTR(true, 16)
  FAP_OUT_FIX_ATTR(false, 16)
  FAP_OUT_FIX_ATTR(true, 32)
  FAP_OUT_FIX_ATTR(false, 32)
#undef FAP_OUT_FIX_ATTR
  return cudaSuccess;
}

cudaError_t launch_sssp(bool f32, const SsspArgs &a, cudaStream_t st) {
  if (a.nbatches <= 0 || a.slots <= 0) return cudaSuccess;
  if (a.lanes != 8 && a.lanes != 16 && a.lanes != 32) return cudaErrorInvalidValue;
  if (a.acc64 && (!f32 || a.lanes == 8)) return cudaErrorInvalidValue;
  if (!(a.delta > 0.0)) return cudaErrorInvalidValue;
  const bool pred = a.pred != nullptr;
  if (f32) return pred ? launch_t<float, true>(a, st) : launch_t<float, false>(a, st);
  return pred ? launch_t<uint32_t, true>(a, st) : launch_t<uint32_t, false>(a, st);
}

cudaError_t launch_sssp_output(bool f32, const SsspArgs &a, cudaStream_t st) {
  if (a.nbatches <= 0) return cudaSuccess;
  if (a.lanes != 8 && a.lanes != 16 && a.lanes != 32) return cudaErrorInvalidValue;
  if ((a.acc64 || a.fix) && (!f32 || a.lanes == 8)) return cudaErrorInvalidValue;
  if (a.fix && a.iwfix == nullptr && a.pred != nullptr) return cudaErrorInvalidValue;
  if (a.slots < a.nbatches) return cudaErrorInvalidValue;
  const bool pred = a.pred != nullptr;
  if (f32) return pred ? launch_output_t<float, true>(a, st) : launch_output_t<float, false>(a, st);
  return pred ? launch_output_t<uint32_t, true>(a, st) : launch_output_t<uint32_t, false>(a, st);
}

int sssp_lanes_for(int64_t batches8, int64_t batches32, int sm_count, bool acc64) {
  // Half-warp batches double the CTA count and the frontier vertices a warp
  // relaxes at once; worth it while 32-source batches leave SMs idle, and
  // quarter-warp batches again while they still fit in one wave.  The
  // FP64 search always takes 16: on the 114,599-vertex road-like graph with
  // 128 parts, 129 batches of 32 in one wave searched in 431 ms against
  // 225 ms for 220 batches of 16 in two waves (one CTA per SM; 179 ms in
  // one wave at two per SM).
  if (acc64) return 16;
  if (batches8 <= sm_count) return 8;
  return batches32 < 2LL * sm_count ? 16 : 32;
}

}  // namespace fapk
