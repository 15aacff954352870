// bgraph.cu -- the boundary SSSP by way of the boundary graph.
//
// Reference counterpart: handle_boundry_path / dijkstra_path
// (fap/kernel/batch_sssp.h:79-114, 280-303): one Dijkstra over the whole
// graph from every boundary vertex.  The rows it produces (distances from
// each boundary vertex to every vertex, and Dijkstra's predecessors) are
// produced here in three steps that never search the whole graph:
//
//   1. local rows: for every part q and every boundary vertex b of q, the
//      distances from b to the vertices of q along edges inside q
//      (L_q[b][v]; bdy_q x sub_q per part), by a frontier Bellman-Ford in
//      shared memory, one CTA per (part, 8 sources);
//   2. boundary graph: its nodes are all boundary vertices, its edges the
//      cut edges (both ends are boundary vertices by the definition of
//      findBoundry, fap/utils/util_preprocess.h:32-58) and, inside every
//      part, b -> b' with weight L_q[b][b'].  A frontier Bellman-Ford in
//      shared memory per 8 sources gives D_S[s][t] for all boundary s, t;
//   3. rows: for v in part q, D[s][v] = min over boundary b of q of
//      D_S[s][b] + L_q[b][v] -- a min-plus per (source batch, part).
//
// Why it is exact: on a shortest path from s to v in part q, the vertex
// after the last cut edge is a boundary vertex b of q and the rest of the
// path stays inside q, so the path is D_S[s][b] + L_q[b][v]; and a shortest
// path between boundary vertices splits at its cut edges into pieces inside
// one part, each no shorter than the L_q entry of its ends.  The arithmetic
// is exact: int32 distances are integers, and FP32 weights are taken as
// 64-bit fixed point (multiples of 2^-shift, where every weight is such a
// multiple and every path length stays below 2^52 units, which the engine
// checks), so every order of additions gives the same numbers -- the
// distances the reference's Dijkstra would compute in exact arithmetic.
//
// Step 3 writes the same vertex-major per-batch tables as the whole-graph
// search (sssp.cu), and the same output pass turns them into rows:
// predecessors by the Dijkstra tie rule from the in-edges (for FP32 graphs
// with integer comparisons in the fixed-point units), rounding (FP32 from the
// fixed point: an exact product by 2^-shift in FP64, then one rounding),
// transposes and coalesced row stores.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "kernels.cuh"
#include "launch.h"

namespace fapk {

namespace {

constexpr int kBgThreads = 512;
constexpr int kBgWarps = kBgThreads / 32;
constexpr int kBgLanes = 8;          // sources per CTA in steps 1 and 2
constexpr int kBgGroups = 32 / kBgLanes;  // frontier nodes a warp relaxes at once
constexpr int kBgEdges = 8;               // edges of a node whose loads are in flight together
constexpr int kRowThreads = 256;     // step 3
constexpr int kRowTA = 32;           // boundary vertices per step-3 chunk

template <typename V>
__host__ __device__ constexpr V bg_inf() {
  return sizeof(V) == 4 ? (V)0x40000000u : (V)(1ull << 62);
}

__device__ __forceinline__ bool bg_set_bit(unsigned *bits, int v) {
  const unsigned m = 1u << (v & 31);
  return (atomicOr(&bits[v >> 5], m) & m) == 0u;
}

// Shared-memory layout of steps 1 and 2 for N nodes: d[N][kBgLanes] (V) |
// list[2][N] | bits[2][words].
template <typename V>
__host__ __device__ inline size_t bg_smem(int N) {
  const size_t words = (size_t)(N + 31) / 32;
  return (size_t)N * kBgLanes * sizeof(V) + (size_t)2 * N * 4 + 2 * words * 4;
}

// Frontier Bellman-Ford over N nodes with kBgLanes sources at once, in
// shared memory.  `relax(u, lane, du, push)` relaxes node u's out-edges for
// one lane (du = that lane's distance of u) and calls push(v, improved) once
// per edge in lockstep across the group's lanes.  The sources' own entries
// were set to 0 and listed by the caller.
//
// With delta > 0 the frontier is worked in distance order, as in
// delta-stepping: a node whose smallest distance over the lanes is above a
// threshold stays in the frontier unrelaxed, and when a round has relaxed
// nothing the threshold moves to the smallest deferred distance + delta.
// Nodes are then relaxed about once each instead of being re-relaxed every
// time a lane improves them (on the boundary graph of the 114,599-vertex
// road-like graph each node was relaxed about ten times).  The order of the
// relaxations never changes the fixpoint the distances converge to.
// Returns false at the round cap.
template <typename V, typename Relax>
__device__ bool bg_bellman_ford(V *d, int *list0, unsigned *bits0, int N, int *s_cnt, V delta, Relax relax,
                                unsigned long long &rounds, unsigned long long &visited) {
  __shared__ int s_done[2];                  // nodes relaxed in the round (by round parity)
  __shared__ unsigned long long s_defer[2];  // smallest deferred distance (by round parity)
  const int words = (N + 31) / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane / kBgLanes, gl = lane % kBgLanes;
  if (threadIdx.x < 2) {
    s_done[threadIdx.x] = 0;
    s_defer[threadIdx.x] = ~0ull;
  }
  __syncthreads();
  V thr = delta;
  int cur = 0;
  for (int r = 0;; r++) {
    const int f = s_cnt[cur];
    if (f == 0) return true;
    // a shortest path has at most N - 1 edges; rounds that only defer
    // alternate with rounds that relax
    if (r > 4 * N + 16) return false;
    rounds++;
    const int par = r & 1;
    const int nxt = cur ^ 1;
    const int *lcur = list0 + cur * N;
    int *lnxt = list0 + nxt * N;
    unsigned *bcur = bits0 + cur * words, *bnxt = bits0 + nxt * words;
    for (int base = warp * kBgGroups; base < f; base += kBgWarps * kBgGroups) {
      const int idx = base + grp;
      int u = idx < f ? lcur[idx] : -1;
      V du = u >= 0 ? d[(size_t)u * kBgLanes + gl] : bg_inf<V>();
      V key = du;
#pragma unroll
      for (int o = 1; o < kBgLanes; o <<= 1) {
        const V other = __shfl_xor_sync(0xffffffffu, key, o);
        key = other < key ? other : key;
      }
      const bool defer = delta > 0 && u >= 0 && key > thr;
      if (u >= 0 && gl == 0) {
        atomicAnd(&bcur[u >> 5], ~(1u << (u & 31)));
        if (defer) {
          if (bg_set_bit(bnxt, u)) lnxt[atomicAdd(&s_cnt[nxt], 1)] = u;
          atomicMin(&s_defer[par], (unsigned long long)key);
        } else {
          atomicAdd(&s_done[par], 1);
        }
      }
      if (defer) u = -1;
      if (u >= 0) visited++;
      relax(u, gl, u >= 0 ? du : bg_inf<V>(), [&](int v, bool improved) {
        // one lane of the group files v when any lane improved it
        const unsigned bal = __ballot_sync(0xffffffffu, improved);
        const unsigned gmask = ((1u << kBgLanes) - 1u) << (grp * kBgLanes);
        if (gl == 0 && (bal & gmask) && bg_set_bit(bnxt, v)) lnxt[atomicAdd(&s_cnt[nxt], 1)] = v;
      });
    }
    __syncthreads();
    if (delta > 0 && s_done[par] == 0) thr = (V)s_defer[par] + delta;  // nothing was below it
    if (threadIdx.x == 0) {
      s_cnt[cur] = 0;
      s_done[par ^ 1] = 0;  // last read in the previous round
      s_defer[par ^ 1] = ~0ull;
    }
    cur = nxt;
    __syncthreads();
  }
}

template <typename V>
__device__ __forceinline__ bool bg_try(V *slot, V c) {
  if (c >= *slot) return false;
  return c < atomicMin(slot, c);
}

// Step 1: local rows.  Job = (part, first local boundary index, count).
template <typename V>
__global__ void __launch_bounds__(kBgThreads) bg_local_kernel(BgArgs a) {
  extern __shared__ __align__(16) unsigned char bg_smem_raw[];
  __shared__ int s_cnt[2];
  const BgJob job = a.ljobs[blockIdx.x];
  const BgPart q = a.parts[job.unit];
  const int N = q.sub;
  V *d = reinterpret_cast<V *>(bg_smem_raw);
  int *list0 = reinterpret_cast<int *>(d + (size_t)N * kBgLanes);
  unsigned *bits0 = reinterpret_cast<unsigned *>(list0 + 2 * N);
  const int words = (N + 31) / 32;
  for (int i = threadIdx.x; i < N * kBgLanes; i += blockDim.x) d[i] = bg_inf<V>();
  for (int i = threadIdx.x; i < 2 * words; i += blockDim.x) bits0[i] = 0u;
  if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  if (threadIdx.x < job.count) {
    const int s = job.first + threadIdx.x;  // local index of the source (boundary vertices come first)
    d[(size_t)s * kBgLanes + threadIdx.x] = 0;
    bg_set_bit(bits0, s);
    list0[atomicAdd(&s_cnt[0], 1)] = s;
  }
  __syncthreads();
  const int32_t *lro = a.lro + q.start;
  const V *lw = static_cast<const V *>(a.lw);
  const int lane = threadIdx.x & 31;
  unsigned long long rounds = 0, visited = 0;
  const bool ok = bg_bellman_ford<V>(
      d, list0, bits0, N, s_cnt, (V)a.delta_local,
      [&](int u, int gl, V du, auto push) {
        int e0 = 0, deg = 0;
        if (u >= 0) {
          e0 = lro[u];
          deg = lro[u + 1] - e0;
        }
        int dmax = deg;
#pragma unroll
        for (int o = kBgLanes; o < 32; o <<= 1) dmax = max(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        // kBgEdges edges at a time: their loads issue together
        for (int t0 = 0; t0 < dmax; t0 += kBgEdges) {
          int v[kBgEdges];
          V w[kBgEdges];
#pragma unroll
          for (int q = 0; q < kBgEdges; q++) {
            const bool in = t0 + q < deg;
            v[q] = in ? a.lcol[e0 + t0 + q] : 0;
            w[q] = in ? lw[e0 + t0 + q] : bg_inf<V>();
          }
#pragma unroll
          for (int q = 0; q < kBgEdges; q++) {
            if (t0 + q >= dmax) break;  // uniform over the warp
            bool imp = false;
            if (t0 + q < deg && du < bg_inf<V>()) imp = bg_try(&d[(size_t)v[q] * kBgLanes + gl], (V)(du + w[q]));
            push(v[q], imp);
          }
        }
        (void)lane;
      },
      rounds, visited);
  if (!ok && threadIdx.x == 0) atomicOr(a.status, kErrSsspCap);
  // rows L[first + l][0..N) of this part
  V *L = static_cast<V *>(a.L) + q.loff;
  for (int i = threadIdx.x; i < job.count * N; i += blockDim.x) {
    const int l = i / N, v = i - l * N;
    L[(size_t)(job.first + l) * N + v] = d[(size_t)v * kBgLanes + l];
  }
  if (threadIdx.x == 0 && a.stats) {
    atomicAdd(&a.stats[0], rounds);
    atomicAdd(&a.stats[2], visited);
  }
}

// Step 2: boundary graph.  Job = (batch of the solve's SSSP sources, first
// lane, count): sources are the boundary indices a.bsrc[batch][first + l].
template <typename V>
__global__ void __launch_bounds__(kBgThreads) bg_boundary_kernel(BgArgs a) {
  extern __shared__ __align__(16) unsigned char bg_smem_raw[];
  __shared__ int s_cnt[2];
  const BgJob job = a.bjobs[blockIdx.x];
  const int N = a.B;
  V *d = reinterpret_cast<V *>(bg_smem_raw);
  int *list0 = reinterpret_cast<int *>(d + (size_t)N * kBgLanes);
  unsigned *bits0 = reinterpret_cast<unsigned *>(list0 + 2 * N);
  const int words = (N + 31) / 32;
  for (int i = threadIdx.x; i < N * kBgLanes; i += blockDim.x) d[i] = bg_inf<V>();
  for (int i = threadIdx.x; i < 2 * words; i += blockDim.x) bits0[i] = 0u;
  if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const int32_t *srcs = a.bsrc + (size_t)job.unit * 32 + job.first;
  if (threadIdx.x < job.count) {
    const int s = srcs[threadIdx.x];
    if (s >= 0 && s < N) {
      d[(size_t)s * kBgLanes + threadIdx.x] = 0;
      if (bg_set_bit(bits0, s)) list0[atomicAdd(&s_cnt[0], 1)] = s;
    } else {
      atomicOr(a.status, kErrBadInput);
    }
  }
  __syncthreads();
  const V *L = static_cast<const V *>(a.L);
  const V *cw = static_cast<const V *>(a.cw);
  unsigned long long rounds = 0, visited = 0;
  const bool ok = bg_bellman_ford<V>(
      d, list0, bits0, N, s_cnt, (V)a.delta_boundary,
      [&](int u, int gl, V du, auto push) {
        // the node's part-mates (row of its part's local rows), then its cut edges
        int nb = 0, boff = 0, e0 = 0, ncut = 0;
        const V *Lrow = nullptr;
        if (u >= 0) {
          const BgPart q = a.parts[a.bpart[u]];
          nb = q.bdy;
          boff = q.boff;
          Lrow = L + q.loff + (size_t)(u - q.boff) * q.sub;
          e0 = a.cro[u];
          ncut = a.cro[u + 1] - e0;
        }
        int tot = nb + ncut;
        int tmax = tot;
#pragma unroll
        for (int o = kBgLanes; o < 32; o <<= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
        const bool live = du < bg_inf<V>();
        // kBgEdges edges at a time: their loads issue together
        for (int t0 = 0; t0 < tmax; t0 += kBgEdges) {
          int v[kBgEdges];
          V w[kBgEdges];
#pragma unroll
          for (int q = 0; q < kBgEdges; q++) {
            const int t = t0 + q;
            v[q] = 0;
            w[q] = bg_inf<V>();
            if (t < nb) {
              v[q] = boff + t;
              w[q] = Lrow[t];
            } else if (t < tot) {
              v[q] = a.ccol[e0 + t - nb];
              w[q] = cw[e0 + t - nb];
            }
          }
#pragma unroll
          for (int q = 0; q < kBgEdges; q++) {
            if (t0 + q >= tmax) break;  // uniform over the warp
            bool imp = false;
            if (live && t0 + q < tot && v[q] != u && w[q] < bg_inf<V>())
              imp = bg_try(&d[(size_t)v[q] * kBgLanes + gl], (V)(du + w[q]));
            push(v[q], imp);
          }
        }
      },
      rounds, visited);
  if (!ok && threadIdx.x == 0) atomicOr(a.status, kErrSsspCap);
  V *DS = static_cast<V *>(a.DS);
  for (int l = 0; l < job.count; l++) {
    const int s = srcs[l];
    if (s < 0 || s >= N) continue;
    for (int v = threadIdx.x; v < N; v += blockDim.x) DS[(size_t)s * N + v] = d[(size_t)v * kBgLanes + l];
  }
  if (threadIdx.x == 0 && a.stats) {
    atomicAdd(&a.stats[0], rounds);
    atomicAdd(&a.stats[2], visited);
  }
}

template <typename V>
__device__ __forceinline__ V bg_addmin(V x, V y, V acc) {
  if constexpr (sizeof(V) == 4)
    return __viaddmin_u32(x, y, acc);  // DPX: min(x + y, acc)
  else
    return min(x + y, acc);
}

// Step 3: rows of one SSSP batch (LANES sources) over the vertices of one
// part, written into the batch's vertex-major table (slot = batch index):
// D[s][v] = min over the part's boundary b of D_S[s][b] + L_q[b][v].
// A thread owns 4 sources x 4 vertices (16 outputs from 8 shared loads per
// boundary vertex); a pass covers row_pass<LANES>() vertices; the boundary
// goes through in chunks of kRowTA.
// OUT64: table of 64-bit fixed-point values, else uint32.
template <int LANES>
__host__ __device__ constexpr int row_pass() { return (kRowThreads / (LANES / 4)) * 4; }

template <typename V, int LANES>
__host__ __device__ constexpr size_t row_smem() {
  return (size_t)kRowTA * (LANES + row_pass<LANES>()) * sizeof(V);
}

template <typename V, int LANES, bool OUT64>
__global__ void __launch_bounds__(kRowThreads) bg_rows_kernel(BgArgs a, BgRowArgs r) {
  constexpr int LG = LANES / 4;          // lane quads
  constexpr int TJ = row_pass<LANES>();  // vertices per pass
  extern __shared__ __align__(16) unsigned char row_smem_raw[];
  V *s_ds = reinterpret_cast<V *>(row_smem_raw);  // [kRowTA][LANES]
  V *s_l = s_ds + kRowTA * LANES;                 // [kRowTA][TJ]
  const int b = blockIdx.x;
  const BgPart q = a.parts[blockIdx.y];
  const int cnt = r.batches[b].count;
  const int32_t *srcs = a.bsrc + (size_t)b * 32;
  const V *DS = static_cast<const V *>(a.DS);
  const V *L = static_cast<const V *>(a.L) + q.loff;
  using K = typename std::conditional<OUT64, unsigned long long, unsigned>::type;
  K *dvm = reinterpret_cast<K *>(static_cast<unsigned char *>(r.scratch) + (size_t)b * r.slot_bytes);
  const int lq = threadIdx.x % LG, vq = threadIdx.x / LG;  // this thread's lanes 4lq.., vertices 4vq..
  for (int j0 = 0; j0 < q.sub; j0 += TJ) {
    V acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[i][c] = (V)(2 * (unsigned long long)bg_inf<V>());
    for (int a0 = 0; a0 < q.bdy; a0 += kRowTA) {
      const int na = min(kRowTA, q.bdy - a0);
      __syncthreads();
      for (int i = threadIdx.x; i < kRowTA * LANES; i += kRowThreads) {
        const int t = i / LANES, l = i - t * LANES;
        V x = bg_inf<V>();
        if (l < cnt && t < na) {
          const int s = srcs[l];  // -1 (not a boundary vertex) was flagged by step 2
          if (s >= 0 && s < a.B) x = DS[(size_t)s * a.B + q.boff + a0 + t];
        }
        s_ds[i] = x;
      }
      for (int i = threadIdx.x; i < kRowTA * TJ; i += kRowThreads) {
        const int t = i / TJ, jj = i - t * TJ;
        s_l[i] = (t < na && j0 + jj < q.sub) ? L[(size_t)(a0 + t) * q.sub + j0 + jj] : bg_inf<V>();
      }
      __syncthreads();
      for (int t = 0; t < na; t++) {
        V x[4], y[4];
#pragma unroll
        for (int i = 0; i < 4; i++) x[i] = s_ds[t * LANES + lq * 4 + i];
#pragma unroll
        for (int c = 0; c < 4; c++) y[c] = s_l[t * TJ + vq * 4 + c];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int c = 0; c < 4; c++) acc[i][c] = bg_addmin(x[i], y[c], acc[i][c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int jj = vq * 4 + c;
      if (j0 + jj >= q.sub) continue;
      const int v = r.st2ed[q.start + j0 + jj];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int l = lq * 4 + i;
        K out;
        if constexpr (OUT64)  // fixed point as it is (the output pass rounds it)
          out = (l >= cnt || acc[i][c] >= r.fix_inf) ? (K)r.fix_inf : (K)acc[i][c];
        else
          out = (l >= cnt || acc[i][c] >= bg_inf<V>()) ? (K)bg_inf<V>() : (K)acc[i][c];
        dvm[(size_t)v * LANES + l] = out;
      }
    }
  }
}

template <typename V>
cudaError_t set_bg_attrs() {
  cudaError_t e = cudaFuncSetAttribute(bg_local_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kBgSmemMax);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(bg_boundary_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kBgSmemMax);
}

template <typename V, int LANES, bool OUT64>
cudaError_t launch_rows_t(const BgArgs &a, const BgRowArgs &r, cudaStream_t st) {
  const dim3 grid((unsigned)r.nbatches, (unsigned)a.nparts);
  ++launch_count();
  bg_rows_kernel<V, LANES, OUT64><<<grid, kRowThreads, row_smem<V, LANES>(), st>>>(a, r);
  return cudaGetLastError();
}

template <typename V, int LANES, bool OUT64>
cudaError_t set_rows_attr() {
  return cudaFuncSetAttribute(bg_rows_kernel<V, LANES, OUT64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)row_smem<V, LANES>());
}

}  // namespace

size_t bg_smem_bytes(bool wide, int nodes) {
  return wide ? bg_smem<unsigned long long>(nodes) : bg_smem<uint32_t>(nodes);
}
int bg_lanes() { return kBgLanes; }

cudaError_t init_bg_kernels() {
  cudaError_t e;
  if ((e = set_bg_attrs<uint32_t>()) != cudaSuccess || (e = set_bg_attrs<unsigned long long>()) != cudaSuccess ||
      (e = set_rows_attr<unsigned long long, 16, true>()) != cudaSuccess ||
      (e = set_rows_attr<unsigned long long, 32, true>()) != cudaSuccess ||
      (e = set_rows_attr<uint32_t, 8, false>()) != cudaSuccess ||
      (e = set_rows_attr<uint32_t, 16, false>()) != cudaSuccess ||
      (e = set_rows_attr<uint32_t, 32, false>()) != cudaSuccess)
    return e;
  return cudaSuccess;
}

cudaError_t launch_bg_local(bool wide, const BgArgs &a, int njobs, int max_sub, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = bg_smem_bytes(wide, max_sub);
  if (smem > kBgSmemMax) return cudaErrorInvalidValue;
  ++launch_count();
  if (wide)
    bg_local_kernel<unsigned long long><<<njobs, kBgThreads, smem, st>>>(a);
  else
    bg_local_kernel<uint32_t><<<njobs, kBgThreads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_bg_boundary(bool wide, const BgArgs &a, int njobs, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = bg_smem_bytes(wide, a.B);
  if (smem > kBgSmemMax) return cudaErrorInvalidValue;
  ++launch_count();
  if (wide)
    bg_boundary_kernel<unsigned long long><<<njobs, kBgThreads, smem, st>>>(a);
  else
    bg_boundary_kernel<uint32_t><<<njobs, kBgThreads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_bg_rows(bool wide, int lanes, const BgArgs &a, const BgRowArgs &r, cudaStream_t st) {
  if (r.nbatches <= 0 || a.nparts <= 0) return cudaSuccess;
  if (wide) {  // FP32 graphs in fixed point: 8-byte tables (the FP64 search's layout)
    if (lanes == 16) return launch_rows_t<unsigned long long, 16, true>(a, r, st);
    if (lanes == 32) return launch_rows_t<unsigned long long, 32, true>(a, r, st);
    return cudaErrorInvalidValue;
  }
  if (lanes == 8) return launch_rows_t<uint32_t, 8, false>(a, r, st);
  if (lanes == 16) return launch_rows_t<uint32_t, 16, false>(a, r, st);
  if (lanes == 32) return launch_rows_t<uint32_t, 32, false>(a, r, st);
  return cudaErrorInvalidValue;
}

}  // namespace fapk
