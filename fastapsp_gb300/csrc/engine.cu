// engine.cu -- the Fast-APSP engine behind the C ABI (include/fastapsp.h).
//
// Reference counterpart: fapGraph::run / solve / solveSubGraph
// (fap/fap.cpp:195-545).  The reference allocates, copies and frees device
// memory around every phase of every part and synchronizes after each kernel.
// Here the engine keeps the graph, its metadata and all work buffers resident
// on one GPU and runs each phase as one launch over a group of parts:
//   SSSP (all boundary sources of the group) -> build (all part matrices) ->
//   FW rounds (diagonal / panels / remaining tiles) -> min-plus -> decode.
// FAP_MODE_PLAIN uses groups of one part in part order (the reference's host
// loop); FAP_MODE_BATCHED uses one group of all parts and replays the launch
// sequence from a CUDA graph that is captured once per (output, parts) key.
//
// All work tables (segments, jobs, batches) for one solve are built on the
// host, uploaded once and kept with the plan, so a replay reads the same
// device tables.

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "fap_internal.h"
#include "kernels.cuh"
#include "launch.h"

using fapk::FwDiagJob;
using fapk::MpSegment;
using fapk::PartDesc;
using fapk::SsspBatch;

namespace fapi {

namespace {
thread_local std::string g_last_error;
}

int set_error(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}
void clear_error() { g_last_error.clear(); }
const char *last_error() { return g_last_error.c_str(); }

}  // namespace fapi

using fapi::set_error;

#define FAP_CUDA(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return set_error(e_ == cudaErrorMemoryAllocation ? FAP_ERR_NOMEM : FAP_ERR_CUDA, \
                       std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

namespace {

// Device buffer that only grows.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need) {
    if (need <= bytes) return FAP_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return set_error(FAP_ERR_NOMEM, "cudaMalloc of " + std::to_string(need) + " bytes failed");
    }
    bytes = need;
    return FAP_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// A fully prepared launch sequence for a list of part groups.
struct Plan {
  // key
  int mode = -1;
  void *dist = nullptr;
  int32_t *pred = nullptr;
  std::vector<int32_t> parts;
  std::vector<int64_t> row_offs;
  // Boundary rows in their own device buffer (null: in dist/pred with the
  // part's other rows): part i's boundary rows start at element brow_offs[i].
  void *bdist = nullptr;
  int32_t *bpred = nullptr;
  std::vector<int64_t> brow_offs;
  // Page-locked host rows that the plan copies its results to, group by
  // group on the copy stream as each group finishes (null: none).
  void *hdist = nullptr;
  int32_t *hpred = nullptr;
  // Staged host results in two slots of dist/pred (ring_elems elements
  // each): group g computes its rows in slot g % 2, after the copy-out of
  // group g - 2 from that slot (0: every row at its own offset).
  int64_t ring_elems = 0;
  std::vector<const void *> sig;  // engine work buffers the tables point into
  // device tables (one allocation)
  DevBuf tables;
  struct Group {
    // SSSP
    const SsspBatch *batches = nullptr;
    int nbatches = 0;
    // the same sources in batches of the other width (sssp_lanes_alt), for
    // the autotuner; swapped with the above when that width wins
    const SsspBatch *batches_alt = nullptr;
    int nbatches_alt = 0;
    // boundary-graph SSSP: step-2 jobs and each batch's sources as boundary indices
    const fapk::BgJob *bjobs = nullptr;
    int nbjobs = 0;
    const int32_t *bsrc = nullptr;
    // build / decode
    const PartDesc *pdesc = nullptr;
    const int64_t *row_begin = nullptr;
    const int64_t *dec_begin = nullptr;
    int nparts = 0;
    int64_t total_rows = 0;
    int64_t dec_rows = 0;
    // FW: per round r, diag jobs [diag_off[r], +diag_cnt[r]) and segments
    std::vector<const FwDiagJob *> diag;
    std::vector<int> diag_cnt;
    std::vector<const MpSegment *> panel;
    std::vector<int> panel_nseg, panel_tiles;
    std::vector<const MpSegment *> rest;
    std::vector<int> rest_nseg, rest_tiles;
    // lookahead (packed and FP32 forms): the remaining tiles of round r
    // without block row and column r + 1 (which the pivot step or chain of
    // round r + 1 updates itself), strip form
    std::vector<const MpSegment *> rest2;
    std::vector<int> rest2_nseg, rest2_strips;
    // FP32 form: round r's row and column panels, strip form
    std::vector<const MpSegment *> pstrips;
    // FP32 form with lookahead: round r - 1's update of block row and column
    // r (the tiles `rest2` of round r - 1 leaves out), strip form
    std::vector<const MpSegment *> look;
    std::vector<int> look_nseg, look_strips;
    const void *tmaps = nullptr;  // tensor-map pairs of the FW matrices (null: none)
    std::vector<int> pstrips_nseg, pstrips_strips;
    // boundary rows in their own buffer (host results): per part {element
    // offset in the results, element offset in the buffer, elements}, copied
    // out as soon as the SSSP has written them
    std::vector<std::array<int64_t, 3>> bnd_copies;
    // min-plus
    const MpSegment *mp = nullptr;
    int mp_nseg = 0, mp_tiles = 0;
    // strip form: class c (K up to fapk::minplus_strip_class_k(c)) holds
    // mp_cls_nseg[c] segments from mp_cls_first[c], one launch each with CTAs
    // numbered from 0; mp_strip_tiles = tiles of all of them in the tile
    // numbering, which the tile form's launch skips
    static constexpr int kMaxCls = 4;
    int mp_ncls = 0, mp_strip_tiles = 0;
    int mp_cls_first[kMaxCls] = {}, mp_cls_nseg[kMaxCls] = {};
    int mp_cls_strips[kMaxCls] = {}, mp_cls_max_k[kMaxCls] = {};
    int mp_cls_cols[kMaxCls] = {};  // tile columns the tuner chose (0: the class default)
    bool mp_aligned = true;  // every strip segment's result rows start on 16-byte boundaries
    int max_sub = 0;  // largest part of the group (bound of the packed form)
    int64_t out_lo = 0, out_elems = 0;  // the group's result rows: elements [out_lo, out_lo + out_elems)
    int64_t dev_lo = 0;                 // where they are computed in dist/pred (out_lo, or its slot)
  };
  std::vector<Group> groups;
  size_t fw_elems = 0;  // FW arena elements needed
  int max_sub = 0;      // largest part of the plan
  int max_mp_k = 0;     // largest min-plus K (boundary count) of the plan
  int pack = -1;        // packed int32 form: -1 undecided, 0 no, 1 yes
  int sssp_lanes = 32;  // sources per SSSP batch
  int sssp_lanes_alt = 0;  // the other width the autotuner tries (0: none)
  int bsssp = 0;        // boundary SSSP through the boundary graph (bgraph.cu) instead of the search
  bool method_trial = false;  // first run times both SSSP methods (automatic choice)
  // FW add-mins of one run outside the remaining-tile strips: the pivot
  // steps' 64^3 block products (packed form), or every block (tile form)
  unsigned long long fw_pivot_work = 0, fw_tile_work = 0;
  int launches = 0;     // kernels one run of the plan launches
  // graph (batched mode)
  cudaGraphExec_t exec = nullptr;
  ~Plan() {
    if (exec) cudaGraphExecDestroy(exec);
    tables.release();
  }
};

// Host-side table builder: appends POD records into one byte buffer and
// remembers offsets, which become device pointers after the upload.
// Storage of one CUtensorMap (encoded by fapk::encode_fw_tmaps).
struct alignas(64) TmapBlob {
  unsigned char bytes[128];
};

struct TableBuilder {
  std::vector<unsigned char> bytes;
  template <typename T>
  size_t add(const T *data, size_t count) {
    size_t off = align_up(bytes.size(), 64);
    bytes.resize(off + sizeof(T) * count);
    if (count) std::memcpy(bytes.data() + off, data, sizeof(T) * count);
    return off;
  }
};

}  // namespace

struct fap_engine {
  int device = 0;
  bool has_graph = false;
  int dtype = FAP_DTYPE_F32;
  int32_t n = 0;
  int64_t m = 0;
  int32_t K = 0;
  int sm_count = 0;
  std::vector<int32_t> ro, col, graph_id, st2ed, ed2st, ver_num, ver_offset, bdy_num, bdy_offset;
  std::vector<float> w;
  uint32_t wmax = 0;  // largest weight (int32 mode)
  double wmean = 1.0; // mean weight (sets the SSSP near-far step)
  // SSSP options (fap_set_option)
  int sssp_fp64 = 0;       // FP32 engines: search in FP64
  double sssp_delta = 0;   // near-far threshold step; 0 = auto (tuned on first solve)
  int autotune = 1;        // tune the SSSP step on the first solve
  int sssp_lanes = 0;      // sources per SSSP batch: 16, 32, 0 = chosen per solve
  int sssp_lanes_tuned = 0;  // the width the autotuner chose (0: none yet)
  int tile_cols = 0;       // min-plus strip tile columns: 64, 128, 0 = per class
  int host_results = 0;    // FAP_OPT_HOST_RESULTS: 0 staged when the device has room, 1 direct
  double host_group_mb = 8192.0;  // FAP_OPT_HOST_GROUP_MB: result rows per group of a host-results solve
  int int32_form = 0;      // FAP_OPT_INT32_FORM: 0 packed keys when provably exact, 1 always wide
  int sssp_method = 0;     // FAP_OPT_SSSP_METHOD: 0 auto, 1 whole-graph search, 2 boundary graph where exact
  int sssp_method_tuned = 0;  // auto: what the first run's trial chose (1 search, 2 boundary graph)
  int fix_shift = -1;      // FP32 graphs: every weight is a multiple of 2^-fix_shift and every path
                           // length below 2^52 of those units (-1: no such shift)
  // boundary graph (bgraph.cu), built for the current partition on first use
  bool bg_ready = false;
  bool bg_ok = false;      // usable: exact arithmetic and both shared-memory tables fit
  int bg_B = 0, bg_max_sub = 0, bg_nljobs = 0;
  std::vector<int32_t> bg_bidx;  // vertex -> boundary index (-1: inner vertex)
  DevBuf bg_tab, bg_L, bg_DS;
  fapk::BgArgs bg_args{};
  const unsigned long long *bg_iwfix = nullptr;  // FP32: in-edge weights in fixed point (in bg_tab)
  unsigned long long bg_fix_inf = 0;             // FP32: fixed-point value of the unreached sentinel
  double delta_try = 0;    // step under trial while tuning
  double tuned_ms = 0;     // SSSP time of the chosen step during tuning
  // device graph
  int32_t *d_ro = nullptr, *d_col = nullptr, *d_iro = nullptr, *d_icol = nullptr;
  int32_t *d_gid = nullptr, *d_st2ed = nullptr, *d_ed2st = nullptr;
  void *d_w = nullptr, *d_iw = nullptr;
  unsigned *d_status = nullptr;
  unsigned long long *d_stats = nullptr;  // SSSP counters of the last solve
  cudaStream_t stream = nullptr;  // highest priority: the FW lookahead's pivot chain runs here
  cudaStream_t side = nullptr;    // lowest priority: the FW remaining tiles beside that chain
  cudaEvent_t ev[6] = {};
  cudaEvent_t ev_sync[2] = {};
  cudaEvent_t ev_fw[3] = {};      // FW lookahead: [0] after pivot step r, [1 + r % 2] after round r's tiles;
                                  // then [0] / [1] fork and join the min-plus classes
  cudaStream_t copy = nullptr;    // early copy-out of boundary rows (host results)
  cudaEvent_t ev_copy[2] = {};    // [0] SSSP rows written, [1] their copy-out done
  cudaEvent_t ev_slot[2] = {};    // staged host results in two slots: slot s's last copy-out done
  // work buffers
  DevBuf fw_d, fw_p;           // FW matrices arena
  DevBuf sssp_scratch, sssp_bits;
  int sssp_slots_alloc = 0;
  bool sssp_wide = false;       // the scratch holds FP64 32-lane slots
  DevBuf res_d, res_p;         // device results when the caller passes host memory
  DevBuf bnd_d, bnd_p;         // boundary rows when the inner rows go straight to mapped host memory
  DevBuf small;                // tables of standalone calls
  std::vector<std::unique_ptr<Plan>> plans;
  double times[5] = {0, 0, 0, 0, 0};
  unsigned long long fw_host_work = 0;  // fw_pivot_work / fw_tile_work of the runs since the last reset
  int64_t last_launches = 0;  // kernels the last solve launched
  std::mutex mu;

  bool f32() const { return dtype == FAP_DTYPE_F32; }
};

namespace {

double sssp_delta_of(const fap_engine *e) {
  if (e->delta_try > 0) return e->delta_try;
  if (e->sssp_delta > 0) return e->sssp_delta;
  // a few mean edge weights per near-far step (at least one unit for int32)
  double d = 8.0 * e->wmean;
  return e->f32() ? std::max(d, 1e-30) : std::max(1.0, std::floor(d));
}

int max_sssp_slots(fap_engine *e, bool wide = false) {
  // Up to two 512-thread CTAs per SM (the FP64 search runs two, the others
  // one at their register count: further batches wait for a free slot),
  // bounded by a 16 GiB scratch budget.
  int slots = std::max(1, 2 * e->sm_count);
  size_t per = fapk::sssp_slot_bytes(e->n, wide) + fapk::sssp_bits_bytes(e->n);
  size_t budget = (size_t)16 << 30;
  slots = (int)std::max<size_t>(1, std::min<size_t>((size_t)slots, budget / std::max<size_t>(per, 1)));
  return slots;
}

// wide: slots of the FP64 search with 32 lanes (twice the distance table);
// sssp_slots_alloc counts slots of the layout last ensured.
int ensure_sssp_scratch(fap_engine *e, int slots, bool wide = false) {
  if (wide != e->sssp_wide) {
    e->sssp_wide = wide;
    size_t fit = e->sssp_scratch.bytes / fapk::sssp_slot_bytes(e->n, wide);
    if (fapk::sssp_bits_bytes(e->n) > 0) fit = std::min(fit, e->sssp_bits.bytes / fapk::sssp_bits_bytes(e->n));
    e->sssp_slots_alloc = (int)fit;
  }
  if (slots <= e->sssp_slots_alloc) return FAP_OK;
  int st;
  if ((st = e->sssp_scratch.ensure(fapk::sssp_slot_bytes(e->n, wide) * slots)) != FAP_OK) return st;
  if ((st = e->sssp_bits.ensure(std::max<size_t>(fapk::sssp_bits_bytes(e->n) * slots, 4))) != FAP_OK)
    return st;
  e->sssp_slots_alloc = slots;
  return FAP_OK;
}

// Host tables of the boundary graph for the current partition (bgraph.cu):
// the parts, the boundary index of every boundary vertex (boundary vertices
// in sorted order), each part's local CSR by sorted position with targets as
// local indices, the cut edges between boundary vertices, the step-1 jobs,
// and the arenas of the local rows and of the boundary-graph distances.
// Weights are uint32 (int32 graphs) or 64-bit fixed point (FP32 graphs, in
// units of 2^-fix_shift, exact).  Sets bg_ok when the method applies.
// Threshold steps of the boundary-graph Bellman-Ford, in mean edge weights
// (0: plain frontier Bellman-Ford).  Measured on the 114,599-vertex road-like
// graph: the boundary graph with 64 mean weights 16.5 ms of SSSP against 18.7
// with none (4-16 were slower); inside the parts none was fastest.
constexpr double kBgDeltaLocal = 0.0, kBgDeltaBoundary = 64.0;

int prepare_bgraph(fap_engine *e) {
  if (e->bg_ready) return FAP_OK;
  e->bg_ready = true;
  e->bg_ok = false;
  const bool wide = e->f32();
  if (wide && e->fix_shift < 0) return FAP_OK;
  const int32_t n = e->n, K = e->K;
  std::vector<fapk::BgPart> parts(K);
  std::vector<int32_t> bpart;
  e->bg_bidx.assign(n, -1);
  int64_t loff = 0;
  int B = 0, max_sub = 0;
  for (int q = 1; q <= K; q++) {
    fapk::BgPart &P = parts[q - 1];
    P.start = e->ver_offset[q];
    P.sub = e->ver_num[q];
    P.bdy = e->bdy_num[q];
    P.boff = B;
    P.loff = loff;
    loff += (int64_t)P.bdy * P.sub;
    for (int a = 0; a < P.bdy; a++) {
      e->bg_bidx[e->st2ed[P.start + a]] = B + a;
      bpart.push_back(q - 1);
    }
    B += P.bdy;
    max_sub = std::max(max_sub, P.sub);
  }
  e->bg_B = B;
  e->bg_max_sub = max_sub;
  if (B == 0 || fapk::bg_smem_bytes(wide, max_sub) > fapk::kBgSmemMax ||
      fapk::bg_smem_bytes(wide, B) > fapk::kBgSmemMax)
    return FAP_OK;
  auto weight = [&](int64_t j) -> uint64_t {
    return wide ? (uint64_t)std::ldexp((double)e->w[j], e->fix_shift) : (uint64_t)e->w[j];
  };
  std::vector<int32_t> lro(n + 1, 0), lcol, cro(B + 1, 0), ccol;
  std::vector<uint64_t> lw, cw;
  lcol.reserve(e->m);
  lw.reserve(e->m);
  for (int32_t pos = 0; pos < n; pos++) {
    const int32_t v = e->st2ed[pos], q = e->graph_id[v];
    const int32_t start = e->ver_offset[q];
    for (int32_t j = e->ro[v]; j < e->ro[v + 1]; j++) {
      const int32_t u = e->col[j];
      if (e->graph_id[u] == q) {
        lcol.push_back(e->ed2st[u] - start);
        lw.push_back(weight(j));
      } else {  // a cut edge joins two boundary vertices; sorted order = boundary-index order
        const int32_t bv = e->bg_bidx[v], bu = e->bg_bidx[u];
        if (bv < 0 || bu < 0) return set_error(FAP_ERR_STATE, "boundary graph: cut edge at an inner vertex");
        ccol.push_back(bu);
        cw.push_back(weight(j));
        cro[bv + 1]++;
      }
    }
    lro[pos + 1] = (int32_t)lcol.size();
  }
  for (int i = 0; i < B; i++) cro[i + 1] += cro[i];
  // FP32: the in-edge weights in fixed point, in the in-edge CSR's order
  // (counting sort by target, sources ascending, as built at creation), for
  // the output pass's integer comparisons
  std::vector<uint64_t> iwfix;
  if (wide) {
    std::vector<int64_t> fill((size_t)n + 1, 0);
    for (int64_t j = 0; j < e->m; j++) fill[e->col[j] + 1]++;
    for (int32_t i = 0; i < n; i++) fill[i + 1] += fill[i];
    iwfix.resize((size_t)e->m);
    for (int32_t u = 0; u < n; u++)
      for (int32_t j = e->ro[u]; j < e->ro[u + 1]; j++) iwfix[fill[e->col[j]]++] = weight(j);
  }
  std::vector<fapk::BgJob> ljobs;
  for (int q = 0; q < K; q++)
    for (int a0 = 0; a0 < parts[q].bdy; a0 += fapk::bg_lanes())
      ljobs.push_back({q, a0, std::min(fapk::bg_lanes(), parts[q].bdy - a0)});
  e->bg_nljobs = (int)ljobs.size();
  TableBuilder tb;
  const size_t o_parts = tb.add(parts.data(), parts.size());
  const size_t o_bpart = tb.add(bpart.data(), bpart.size());
  const size_t o_lro = tb.add(lro.data(), lro.size());
  const size_t o_lcol = tb.add(lcol.data(), lcol.size());
  const size_t o_cro = tb.add(cro.data(), cro.size());
  const size_t o_ccol = tb.add(ccol.data(), ccol.size());
  const size_t o_ljobs = tb.add(ljobs.data(), ljobs.size());
  const size_t o_iwfix = tb.add(iwfix.data(), iwfix.size());
  size_t o_lw, o_cw;
  if (wide) {
    o_lw = tb.add(lw.data(), lw.size());
    o_cw = tb.add(cw.data(), cw.size());
  } else {
    std::vector<uint32_t> lw32(lw.begin(), lw.end()), cw32(cw.begin(), cw.end());
    o_lw = tb.add(lw32.data(), lw32.size());
    o_cw = tb.add(cw32.data(), cw32.size());
  }
  int rc;
  const size_t vs = wide ? 8 : 4;
  if ((rc = e->bg_tab.ensure(std::max<size_t>(tb.bytes.size(), 64))) != FAP_OK ||
      (rc = e->bg_L.ensure(std::max<size_t>((size_t)loff * vs, 8))) != FAP_OK ||
      (rc = e->bg_DS.ensure((size_t)B * B * vs)) != FAP_OK)
    return rc;
  FAP_CUDA(cudaMemcpy(e->bg_tab.p, tb.bytes.data(), tb.bytes.size(), cudaMemcpyHostToDevice));
  unsigned char *base = static_cast<unsigned char *>(e->bg_tab.p);
  fapk::BgArgs &a = e->bg_args;
  a = fapk::BgArgs{};
  a.nparts = K;
  a.parts = reinterpret_cast<const fapk::BgPart *>(base + o_parts);
  a.B = B;
  a.bpart = reinterpret_cast<const int32_t *>(base + o_bpart);
  a.lro = reinterpret_cast<const int32_t *>(base + o_lro);
  a.lcol = reinterpret_cast<const int32_t *>(base + o_lcol);
  a.lw = base + o_lw;
  a.cro = reinterpret_cast<const int32_t *>(base + o_cro);
  a.ccol = reinterpret_cast<const int32_t *>(base + o_ccol);
  a.cw = base + o_cw;
  a.ljobs = reinterpret_cast<const fapk::BgJob *>(base + o_ljobs);
  a.L = e->bg_L.p;
  a.DS = e->bg_DS.p;
  e->bg_iwfix = wide ? reinterpret_cast<const unsigned long long *>(base + o_iwfix) : nullptr;
  // unreached: at or above the sentinel 1e8 (the FP64 search's rule), or the
  // steps' own infinity, whichever is smaller
  e->bg_fix_inf = wide ? (unsigned long long)std::min(std::ldexp(1e8, e->fix_shift), std::ldexp(1.0, 62)) : 0;
  {
    // threshold steps in the weights' units
    double mean = 0;
    for (int64_t j = 0; j < e->m; j++) mean += (double)weight(j);
    mean = e->m > 0 ? std::max(1.0, mean / (double)e->m) : 1.0;
    a.delta_local = (unsigned long long)(kBgDeltaLocal * mean);
    a.delta_boundary = (unsigned long long)(kBgDeltaBoundary * mean);
  }
  e->bg_ok = true;
  return FAP_OK;
}

bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes attr;
  cudaError_t err = cudaPointerGetAttributes(&attr, p);
  if (err != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

// FW segments of one matrix for pivot block r (row panel + column panel, and
// the remaining tiles).  Matrices are size x size with leading dimension ld.
void fw_segments(void *D, int32_t *P, int64_t ld, int size, int r, MpSegment &rowp,
                 MpSegment &colp, MpSegment &rest, int &t_rowp, int &t_colp, int &t_rest,
                 bool f32, int32_t tmap1 = 0) {
  const int B = fapk::fw_block();
  const int nb = (size + B - 1) / B;
  const size_t es = 4;
  (void)f32;
  MpSegment s{};
  s.tmap1 = tmap1;  // the strips' bulk tensor copies, when the matrix has a map pair
  s.b_row0 = r * B;
  s.A = static_cast<const unsigned char *>(D) + (size_t)r * B * es;
  s.lda = ld;
  s.B = static_cast<const unsigned char *>(D) + (size_t)r * B * ld * es;
  s.ldb = ld;
  s.Bp = P ? P + (size_t)r * B * ld : nullptr;
  s.ldbp = ld;
  s.C = D;
  s.ldc = ld;
  s.Cp = P;
  s.ldcp = ld;
  s.M = size;
  s.N = size;
  s.K = std::min(B, size - r * B);
  s.init_from_c = 1;
  const int others = nb - 1;
  const int pairs = (others + 1) / 2;
  rowp = s;
  rowp.row_skip = -1;
  rowp.row_fix = r;
  rowp.col_skip = r;
  rowp.col_fix = -1;
  rowp.tiles_x = pairs;
  t_rowp = pairs;
  colp = s;
  colp.row_skip = r;
  colp.row_fix = -1;
  colp.col_skip = -1;
  colp.col_fix = r;
  colp.tiles_x = 1;
  t_colp = pairs;
  rest = s;
  rest.row_skip = r;
  rest.row_fix = -1;
  rest.col_skip = r;
  rest.col_fix = -1;
  rest.tiles_x = pairs;
  t_rest = pairs * pairs;
}

// CTAs of an FW segment in the strip form (tiles_y row tiles).
int fw_strips_of(const MpSegment &s, int tiles_y) {
  const int T = fapk::fw_strip_tiles();
  return tiles_y * ((s.tiles_x + T - 1) / T);
}

// FP32 form: fw_segments' two panels of pivot block r of nb as strip-form
// segments, appended to `out` from CTA `strips` on.  Each reads and writes
// the same entries (the row panel is B and C, the column panel A and C); a
// CTA reads the entries it writes into shared memory before its epilogue,
// and no two CTAs write the same entries.
void fw_panel_strips(const MpSegment &rowp, const MpSegment &colp, int nb, std::vector<MpSegment> &out,
                     int &strips) {
  MpSegment a = rowp, c = colp;
  a.strip_begin = strips;
  strips += fw_strips_of(rowp, 1);
  out.push_back(a);
  c.strip_begin = strips;
  strips += fw_strips_of(colp, nb / 2);  // (nb - 1) row blocks in pairs
  out.push_back(c);
}

// Lookahead form of fw_segments' `rest` for pivot block r of nb: the rows and
// columns other than r and r + 1 (block row and column r + 1 get round r's
// update inside pivot step r + 1).  Returns its CTAs in the strip form.
int fw_rest_lookahead(MpSegment &rest, int nb, int r) {
  const int pairs = (nb - 2 + 1) / 2;
  rest.row_skip2 = r + 1;
  rest.col_skip2 = r + 1;
  rest.tiles_x = pairs;
  return fw_strips_of(rest, pairs);
}

// FP32 form with lookahead: round r - 1's update of block row and column r
// of nb (r >= 1; the tiles that fw_rest_lookahead leaves out of round
// r - 1) as strip-form segments appended to `out` from CTA `strips` on:
// block row r over the columns other than r - 1 (the pivot block (r, r)
// with them), and block column r over the rows other than r - 1 and r.  The
// two write disjoint blocks and read block row and column r - 1 only, which
// neither writes; no tile reads entries it or another tile writes.
void fw_look_strips(void *D, int32_t *P, int64_t ld, int size, int r, int nb, int32_t tmap1,
                    std::vector<MpSegment> &out, int &strips) {
  MpSegment rowp, colp, rest;
  int t1, t2, t3;
  fw_segments(D, P, ld, size, r - 1, rowp, colp, rest, t1, t2, t3, true, tmap1);
  rowp.row_fix = r;  // (the row panel of pivot r - 1, moved to block row r)
  rowp.strip_begin = strips;
  strips += fw_strips_of(rowp, 1);
  out.push_back(rowp);
  if (nb > 2) {
    colp.col_fix = r;  // (the column panel, moved to block column r, without row r)
    colp.row_skip2 = r;
    colp.strip_begin = strips;
    strips += fw_strips_of(colp, (nb - 1) / 2);  // (nb - 2) row blocks in pairs
    out.push_back(colp);
  }
}

// Min-plus segment C = A (x) B (fresh C), tiled in 128x128.
MpSegment mp_segment(const void *A, int64_t lda, const void *B, int64_t ldb, const int32_t *Bp,
                     int64_t ldbp, void *C, int64_t ldc, int32_t *Cp, int64_t ldcp, int M, int N,
                     int K, int &tiles) {
  MpSegment s{};
  s.A = A;
  s.lda = lda;
  s.B = B;
  s.ldb = ldb;
  s.Bp = Bp;
  s.ldbp = ldbp;
  s.C = C;
  s.ldc = ldc;
  s.Cp = Cp;
  s.ldcp = ldcp;
  s.M = M;
  s.N = N;
  s.K = K;
  s.row_skip = s.col_skip = s.row_fix = s.col_fix = -1;
  s.init_from_c = 0;
  const int T = fapk::minplus_tile_rows();
  s.tiles_x = (N + T - 1) / T;
  tiles = ((M + T - 1) / T) * s.tiles_x;
  return s;
}

// Whether a min-plus segment's result rows (and predecessor rows) all start
// on 16-byte boundaries.
bool rows_aligned16(const MpSegment &s) {
  const bool c = (s.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(s.C) & 15) == 0;
  return c && (s.Cp == nullptr || ((s.ldcp & 3) == 0 && (reinterpret_cast<uintptr_t>(s.Cp) & 15) == 0));
}

// CTAs of a segment in the tile form of the min-plus (no skipped blocks).
int mp_tiles_of(const MpSegment &s) {
  const int T = fapk::minplus_tile_rows();
  return ((s.M + T - 1) / T) * s.tiles_x;
}

// CTAs of a segment in the strip form of the min-plus.
int mp_strips_of(const MpSegment &s) {
  const int T = fapk::minplus_tile_rows(), S = fapk::minplus_strip_tiles();
  return ((s.M + T - 1) / T) * ((s.tiles_x + S - 1) / S);
}

// Groups of a batched plan whose results are copied to host rows:
// consecutive parts (indices into `parts`) in groups of about 8 GB of rows
// (at most 8 groups), so that the copy of one group's rows runs while the
// next group computes.
std::vector<std::vector<int>> host_groups(const fap_engine *e, const std::vector<int32_t> &parts,
                                          bool pred) {
  std::vector<std::vector<int>> groups;
  int64_t rows = 0;
  for (int p : parts) rows += e->ver_num[p];
  const double bytes = (double)rows * e->n * 4 * (pred ? 2 : 1);
  const int ng = (int)std::min<double>(8.0, std::max(1.0, std::ceil(bytes / (e->host_group_mb * (1 << 20)))));
  const int64_t per = (rows + ng - 1) / ng;
  int64_t acc = 0;
  groups.emplace_back();
  for (size_t i = 0; i < parts.size(); i++) {
    if (acc >= per * (int64_t)groups.size() && !groups.back().empty()) groups.emplace_back();
    groups.back().push_back((int)i);
    acc += e->ver_num[parts[i]];
  }
  return groups;
}

// Builds the plan for `parts` (row offsets into dist/pred given per part),
// grouped one part per group (plain) or all in one group (batched).
int build_plan(fap_engine *e, Plan &pl) {
  const bool batched = pl.mode == FAP_MODE_BATCHED;
  const int B = fapk::fw_block();
  const int64_t n = e->n;
  std::vector<std::vector<int>> groups;
  if (batched && pl.hdist) {
    groups = host_groups(e, pl.parts, pl.pred != nullptr);
  } else if (batched) {
    groups.emplace_back();
    for (size_t i = 0; i < pl.parts.size(); i++) groups[0].push_back((int)i);
  } else {
    for (size_t i = 0; i < pl.parts.size(); i++) groups.push_back({(int)i});
  }
  // FW arena layout: every part of the plan gets its own matrix.
  std::vector<int64_t> mat_off(pl.parts.size());
  std::vector<int32_t> ldv(pl.parts.size());
  size_t arena = 0;
  for (size_t i = 0; i < pl.parts.size(); i++) {
    int p = pl.parts[i];
    int sub = e->ver_num[p];
    int ld = sub > 0 ? (int)align_up((size_t)sub, (size_t)B) : 0;
    ldv[i] = ld;
    mat_off[i] = (int64_t)arena;
    arena += (size_t)ld * ld;
  }
  pl.fw_elems = arena;
  char *fwd = static_cast<char *>(e->fw_d.p);
  int32_t *fwp = static_cast<int32_t *>(e->fw_p.p);
  const bool pred = pl.pred != nullptr;
  char *dist = static_cast<char *>(pl.dist);
  // where the boundary rows live: their own buffer, or the part's rows
  char *bdist = pl.bdist ? static_cast<char *>(pl.bdist) : dist;
  int32_t *bpred = pl.bdist ? pl.bpred : pl.pred;

  TableBuilder tb;
  struct GroupOffs {
    size_t batches, batches_alt, pdesc, row_begin, dec_begin, mp, bjobs, bsrc;
    std::vector<size_t> diag, panel, rest, rest2, pstrips, look;
    size_t tmaps = 0;
    bool has_tmaps = false;
  };
  std::vector<GroupOffs> goffs(groups.size());
  pl.groups.assign(groups.size(), Plan::Group{});
  for (size_t g = 0; g < groups.size(); g++) {
    Plan::Group &G = pl.groups[g];
    GroupOffs &O = goffs[g];
    // SSSP batches: per part, its boundary vertices in mapping order.
    std::vector<SsspBatch> batches, batches_alt;
    std::vector<PartDesc> pdesc;
    std::vector<int64_t> row_begin(1, 0), dec_begin(1, 0);
    // min-plus segments: the strip form's classes of K in order, then those
    // above its limit; tiles are numbered over all of them
    std::vector<MpSegment> mps_cls[Plan::Group::kMaxCls], mps_wide;
    const int ncls = std::min(fapk::minplus_strip_classes(), (int)Plan::Group::kMaxCls);
    int maxnb = 0;
    {
      const int first = groups[g].front(), last = groups[g].back();
      G.out_lo = pl.row_offs[first];
      G.out_elems = pl.row_offs[last] + (int64_t)e->ver_num[pl.parts[last]] * n - G.out_lo;
      G.dev_lo = pl.ring_elems > 0 ? (int64_t)(g & 1) * pl.ring_elems : G.out_lo;
    }
    for (int idx : groups[g]) {
      int p = pl.parts[idx];
      int sub = e->ver_num[p], bdy = e->bdy_num[p], start = e->ver_offset[p];
      int64_t roff = pl.row_offs[idx] - G.out_lo + G.dev_lo;  // the part's rows in dist/pred
      int64_t boff = pl.bdist ? pl.brow_offs[idx] : roff;  // first boundary row
      for (int w = 0; w < 2; w++) {
        const int L = w == 0 ? pl.sssp_lanes : pl.sssp_lanes_alt;
        for (int b0 = 0; L > 0 && b0 < bdy; b0 += L) {
          SsspBatch sb{};
          sb.count = std::min(L, bdy - b0);
          for (int l = 0; l < sb.count; l++) {
            sb.src[l] = e->st2ed[start + b0 + l];
            sb.row_off[l] = boff + (int64_t)(b0 + l) * n;
          }
          (w == 0 ? batches : batches_alt).push_back(sb);
        }
      }
      if (sub == 0) continue;
      G.max_sub = std::max(G.max_sub, sub);
      PartDesc d{};
      d.sub = sub;
      d.bdy = bdy;
      d.start = start;
      d.ld = ldv[idx];
      d.mat_off = mat_off[idx];
      d.row_off = boff;
      d.dec_off = roff;  // the decode writes the result rows themselves
      pdesc.push_back(d);
      if (pl.bdist && bdy > 0) G.bnd_copies.push_back({roff, boff, (int64_t)bdy * n});
      row_begin.push_back(row_begin.back() + d.ld);
      dec_begin.push_back(dec_begin.back() + bdy);
      pl.max_sub = std::max(pl.max_sub, sub);
      maxnb = std::max(maxnb, d.ld / B);
      // min-plus for the inner rows
      int inner = sub - bdy;
      if (inner > 0) {
        int tiles = 0;
        const size_t es = 4;
        MpSegment s = mp_segment(fwd + (size_t)(mat_off[idx] + (int64_t)bdy * d.ld) * es, d.ld,
                                 bdist + (size_t)boff * es, n, pred ? bpred + boff : nullptr, n,
                                 dist + (size_t)(roff + (int64_t)bdy * n) * es, n,
                                 pred ? pl.pred + roff + (int64_t)bdy * n : nullptr, n, inner,
                                 (int)n, bdy, tiles);
        // the part's own columns come from the FW matrix (rows bdy..sub-1)
        s.col_part = e->d_gid;
        s.part = p;
        s.col_local = e->d_ed2st;
        s.local0 = start;
        s.F = fwd + (size_t)(mat_off[idx] + (int64_t)bdy * d.ld) * es;
        s.Fp = pred ? fwp + mat_off[idx] + (int64_t)bdy * d.ld : nullptr;
        s.ldf = d.ld;
        pl.max_mp_k = std::max(pl.max_mp_k, bdy);
        int c = 0;
        while (c < ncls && bdy > fapk::minplus_strip_class_k(c)) c++;
        if (n >= (1 << 24)) c = ncls;  // the strip form needs leading dimensions below 2^24
        if (c < ncls) mps_cls[c].push_back(s);
        else mps_wide.push_back(s);
      }
    }
    G.nbatches = (int)batches.size();
    O.batches = tb.add(batches.data(), batches.size());
    if (pl.bsssp) {  // boundary-graph SSSP: each batch's sources as boundary indices, step-2 jobs
      std::vector<int32_t> bsrc((size_t)batches.size() * 32, -1);
      std::vector<fapk::BgJob> bjobs;
      for (size_t b = 0; b < batches.size(); b++) {
        for (int l = 0; l < batches[b].count; l++) bsrc[b * 32 + l] = e->bg_bidx[batches[b].src[l]];
        for (int l0 = 0; l0 < batches[b].count; l0 += fapk::bg_lanes())
          bjobs.push_back({(int32_t)b, l0, std::min(fapk::bg_lanes(), batches[b].count - l0)});
      }
      G.nbjobs = (int)bjobs.size();
      O.bjobs = tb.add(bjobs.data(), bjobs.size());
      O.bsrc = tb.add(bsrc.data(), bsrc.size());
    }
    G.nbatches_alt = (int)batches_alt.size();
    O.batches_alt = tb.add(batches_alt.data(), batches_alt.size());
    G.nparts = (int)pdesc.size();
    G.total_rows = row_begin.back();
    G.dec_rows = dec_begin.back();
    O.pdesc = tb.add(pdesc.data(), pdesc.size());
    O.row_begin = tb.add(row_begin.data(), row_begin.size());
    O.dec_begin = tb.add(dec_begin.data(), dec_begin.size());
    std::vector<MpSegment> mps;
    G.mp_ncls = ncls;
    for (int c = 0; c < ncls; c++) {
      G.mp_cls_first[c] = (int)mps.size();
      G.mp_cls_nseg[c] = (int)mps_cls[c].size();
      for (MpSegment &s : mps_cls[c]) {
        s.strip_begin = G.mp_cls_strips[c];
        G.mp_cls_strips[c] += mp_strips_of(s);
        G.mp_cls_max_k[c] = std::max(G.mp_cls_max_k[c], s.K);
        G.mp_aligned = G.mp_aligned && rows_aligned16(s);
      }
      mps.insert(mps.end(), mps_cls[c].begin(), mps_cls[c].end());
    }
    const int nstrip = (int)mps.size();
    mps.insert(mps.end(), mps_wide.begin(), mps_wide.end());
    int mp_tiles = 0;
    for (MpSegment &s : mps) {
      s.tile_begin = mp_tiles;
      mp_tiles += mp_tiles_of(s);
      if (&s - mps.data() + 1 == nstrip) G.mp_strip_tiles = mp_tiles;
    }
    G.mp_nseg = (int)mps.size();
    G.mp_tiles = mp_tiles;
    O.mp = tb.add(mps.data(), mps.size());
    // FW rounds
    G.diag_cnt.assign(maxnb, 0);
    G.panel_nseg.assign(maxnb, 0);
    G.panel_tiles.assign(maxnb, 0);
    G.rest_nseg.assign(maxnb, 0);
    G.rest_tiles.assign(maxnb, 0);
    G.rest2_nseg.assign(maxnb, 0);
    G.rest2_strips.assign(maxnb, 0);
    G.pstrips_nseg.assign(maxnb, 0);
    G.pstrips_strips.assign(maxnb, 0);
    O.pstrips.assign(maxnb, 0);
    G.look_nseg.assign(maxnb, 0);
    G.look_strips.assign(maxnb, 0);
    O.look.assign(maxnb, 0);
    O.diag.assign(maxnb, 0);
    O.panel.assign(maxnb, 0);
    O.rest.assign(maxnb, 0);
    O.rest2.assign(maxnb, 0);
    // Tensor-map pairs (distances, predecessors) of the parts' FW matrices
    // for the strips' bulk tensor copies; a part without one (no encoder)
    // keeps the per-thread copies.
    std::vector<int32_t> tmap1(pdesc.size(), 0);
    {
      std::vector<TmapBlob> maps;
      for (size_t i = 0; i < pdesc.size(); i++) {
        const PartDesc &d = pdesc[i];
        TmapBlob two[2];
        if (fapk::encode_fw_tmaps(two, fwd + (size_t)d.mat_off * 4, pred ? fwp + d.mat_off : nullptr, d.ld,
                                  d.ld, d.ld)) {
          tmap1[i] = (int32_t)(maps.size() / 2) + 1;
          maps.push_back(two[0]);
          maps.push_back(two[1]);
        }
      }
      if (!maps.empty()) {
        O.tmaps = tb.add(maps.data(), maps.size());
        O.has_tmaps = true;
      }
    }
    for (int r = 0; r < maxnb; r++) {
      std::vector<FwDiagJob> dj;
      std::vector<MpSegment> ps, rs, r2s, pss, ls;
      int pt = 0, rt = 0, r2strips = 0, psstrips = 0, lstrips = 0;
      for (size_t pi = 0; pi < pdesc.size(); pi++) {
        const PartDesc &d = pdesc[pi];
        int nb = d.ld / B;
        if (r >= nb) continue;
        void *D = fwd + (size_t)d.mat_off * 4;
        int32_t *P = pred ? fwp + d.mat_off : nullptr;
        FwDiagJob j{};
        j.D = D;
        j.P = P;
        j.ld = d.ld;
        j.size = d.ld;
        j.block = r;
        j.prev = r - 1;  // used by the packed form's pivot step (lookahead) only
        dj.push_back(j);
        {  // 64^3 block products: pivot step (lookahead update, closure, panels); tile form (all blocks)
          const unsigned long long blk = (unsigned long long)B * B * B;
          pl.fw_pivot_work += blk * ((r > 0 ? 2ull * (nb - 2) + 1 : 0ull) + 1ull + 2ull * (nb - 1));
          pl.fw_tile_work += blk * (e->f32() ? 1ull : (unsigned long long)nb * nb);
        }
        if (nb > 1) {
          MpSegment rp, cp, rest;
          int a1, a2, a3;
          fw_segments(D, P, d.ld, d.ld, r, rp, cp, rest, a1, a2, a3, e->f32(), tmap1[pi]);
          if (e->f32() && r > 0) fw_look_strips(D, P, d.ld, d.ld, r, nb, tmap1[pi], ls, lstrips);
          rp.tile_begin = pt;
          pt += a1;
          ps.push_back(rp);
          cp.tile_begin = pt;
          pt += a2;
          ps.push_back(cp);
          rest.tile_begin = rt;
          rt += a3;
          rs.push_back(rest);
          fw_panel_strips(rp, cp, nb, pss, psstrips);
          MpSegment rest2 = rest;
          const int s2 = r + 1 < nb ? fw_rest_lookahead(rest2, nb, r) : fw_strips_of(rest, rest.tiles_x);
          if (s2 > 0) {
            rest2.strip_begin = r2strips;
            r2strips += s2;
            r2s.push_back(rest2);
          }
        }
      }
      G.diag_cnt[r] = (int)dj.size();
      O.diag[r] = tb.add(dj.data(), dj.size());
      G.panel_nseg[r] = (int)ps.size();
      G.panel_tiles[r] = pt;
      O.panel[r] = tb.add(ps.data(), ps.size());
      G.rest_nseg[r] = (int)rs.size();
      G.rest_tiles[r] = rt;
      O.rest[r] = tb.add(rs.data(), rs.size());
      G.rest2_nseg[r] = (int)r2s.size();
      G.rest2_strips[r] = r2strips;
      O.rest2[r] = tb.add(r2s.data(), r2s.size());
      G.pstrips_nseg[r] = (int)pss.size();
      G.pstrips_strips[r] = psstrips;
      O.pstrips[r] = tb.add(pss.data(), pss.size());
      G.look_nseg[r] = (int)ls.size();
      G.look_strips[r] = lstrips;
      O.look[r] = tb.add(ls.data(), ls.size());
    }
  }
  int st = pl.tables.ensure(std::max<size_t>(tb.bytes.size(), 64));
  if (st != FAP_OK) return st;
  FAP_CUDA(cudaMemcpy(pl.tables.p, tb.bytes.data(), tb.bytes.size(), cudaMemcpyHostToDevice));
  unsigned char *base = static_cast<unsigned char *>(pl.tables.p);
  for (size_t g = 0; g < groups.size(); g++) {
    Plan::Group &G = pl.groups[g];
    GroupOffs &O = goffs[g];
    G.batches = reinterpret_cast<const SsspBatch *>(base + O.batches);
    G.batches_alt = reinterpret_cast<const SsspBatch *>(base + O.batches_alt);
    if (pl.bsssp) {
      G.bjobs = reinterpret_cast<const fapk::BgJob *>(base + O.bjobs);
      G.bsrc = reinterpret_cast<const int32_t *>(base + O.bsrc);
    }
    G.pdesc = reinterpret_cast<const PartDesc *>(base + O.pdesc);
    G.row_begin = reinterpret_cast<const int64_t *>(base + O.row_begin);
    G.dec_begin = reinterpret_cast<const int64_t *>(base + O.dec_begin);
    G.mp = reinterpret_cast<const MpSegment *>(base + O.mp);
    G.tmaps = O.has_tmaps ? static_cast<const void *>(base + O.tmaps) : nullptr;
    size_t R = O.diag.size();
    G.diag.resize(R);
    G.panel.resize(R);
    G.rest.resize(R);
    G.rest2.resize(R);
    G.pstrips.resize(R);
    G.look.resize(R);
    for (size_t r = 0; r < R; r++) {
      G.diag[r] = reinterpret_cast<const FwDiagJob *>(base + O.diag[r]);
      G.panel[r] = reinterpret_cast<const MpSegment *>(base + O.panel[r]);
      G.rest[r] = reinterpret_cast<const MpSegment *>(base + O.rest[r]);
      G.rest2[r] = reinterpret_cast<const MpSegment *>(base + O.rest2[r]);
      G.pstrips[r] = reinterpret_cast<const MpSegment *>(base + O.pstrips[r]);
      G.look[r] = reinterpret_cast<const MpSegment *>(base + O.look[r]);
    }
  }
  return FAP_OK;
}

fapk::BuildArgs build_args(fap_engine *e, const Plan &pl, const Plan::Group &G) {
  fapk::BuildArgs a{};
  a.n = e->n;
  a.ro = e->d_ro;
  a.col = e->d_col;
  a.w = e->d_w;
  a.graph_id = e->d_gid;
  a.st2ed = e->d_st2ed;
  a.ed2st = e->d_ed2st;
  a.parts = G.pdesc;
  a.row_begin = G.row_begin;
  a.dec_begin = G.dec_begin;
  a.nparts = G.nparts;
  a.total_rows = G.total_rows;
  a.dec_rows = G.dec_rows;
  a.mat = e->fw_d.p;
  a.matp = pl.pred ? static_cast<int32_t *>(e->fw_p.p) : nullptr;
  a.rows = pl.bdist ? pl.bdist : pl.dist;  // the boundary rows
  a.rowsp = pl.bdist ? pl.bpred : pl.pred;
  a.ldr = e->n;
  return a;
}

// Launch helpers for one plan.  Phase A is the SSSP of one group, phase B
// the rest of the group (build, FW rounds, min-plus, decode).  Events
// ev[0..5] bracket the phases: ev0 before the first SSSP, ev1 after the last
// SSSP, ev2..ev5 after build / FW / min-plus / decode of the last group.
struct Issuer {
  fap_engine *e;
  Plan &pl;
  cudaStream_t st;
  bool capturing;
  cudaError_t rec(int i) {
    return capturing ? cudaEventRecordWithFlags(e->ev[i], st, cudaEventRecordExternal)
                     : cudaEventRecord(e->ev[i], st);
  }
  int sssp(size_t g) {
    Plan::Group &G = pl.groups[g];
    fapk::SsspArgs sa{};
    sa.n = e->n;
    sa.ro = e->d_ro;
    sa.col = e->d_col;
    sa.w = e->d_w;
    sa.iro = e->d_iro;
    sa.icol = e->d_icol;
    sa.iw = e->d_iw;
    sa.batches = G.batches;
    sa.nbatches = G.nbatches;
    sa.dist = pl.bdist ? pl.bdist : pl.dist;  // SSSP rows are the boundary rows
    sa.pred = pl.bdist ? pl.bpred : pl.pred;
    sa.scratch = e->sssp_scratch.p;
    sa.slots = std::min(G.nbatches, e->sssp_slots_alloc);
    sa.bits = e->sssp_bits.p;
    sa.status = e->d_status;
    sa.maxd = e->f32() ? nullptr : e->d_status + 1;
    sa.iter_cap = 8 * e->n + 64;
    sa.lanes = pl.sssp_lanes;
    sa.acc64 = e->f32() && e->sssp_fp64;
    sa.delta = sssp_delta_of(e);
    sa.stats = e->d_stats;
    if (g == 0) FAP_CUDA(cudaMemsetAsync(e->d_stats, 0, 8 * sizeof(unsigned long long), st));
    if (pl.bsssp) {
      // Through the boundary graph: local rows of every part (once per
      // solve), boundary-graph distances of this group's sources, their
      // rows into the per-batch tables, then the search's output pass.
      const bool wide = e->f32();
      fapk::BgArgs ba = e->bg_args;
      ba.bjobs = G.bjobs;
      ba.bsrc = G.bsrc;
      ba.status = e->d_status;
      ba.stats = e->d_stats;
      if (g == 0) FAP_CUDA(fapk::launch_bg_local(wide, ba, e->bg_nljobs, e->bg_max_sub, st));
      FAP_CUDA(fapk::launch_bg_boundary(wide, ba, G.nbjobs, st));
      fapk::BgRowArgs ra{};
      ra.batches = G.batches;
      ra.nbatches = G.nbatches;
      ra.st2ed = e->d_st2ed;
      ra.scratch = e->sssp_scratch.p;
      ra.slot_bytes = fapk::sssp_slot_bytes(e->n, sa.acc64 && sa.lanes == 32);
      ra.fix_inf = e->bg_fix_inf;
      FAP_CUDA(fapk::launch_bg_rows(wide, sa.lanes, ba, ra, st));
      sa.slots = G.nbatches;
      if (wide) {  // fixed-point tables: integer comparisons, one rounding
        sa.fix = 1;
        sa.acc64 = 0;
        sa.iwfix = e->bg_iwfix;
        sa.fix_inf = e->bg_fix_inf;
        sa.fix_scale = std::ldexp(1.0, -e->fix_shift);
      }
      FAP_CUDA(fapk::launch_sssp_output(e->f32(), sa, st));
      return FAP_OK;
    }
    FAP_CUDA(fapk::launch_sssp(e->f32(), sa, st));
    return FAP_OK;
  }
  int rest(size_t g, bool last) {
    const bool f32 = e->f32();
    const bool pred = pl.pred != nullptr;
    const bool packed = pl.pack == 1;
    Plan::Group &G = pl.groups[g];
    fapk::BuildArgs ba = build_args(e, pl, G);
    FAP_CUDA(fapk::launch_build(f32, pred, ba, st));
    if (!G.bnd_copies.empty()) {
      // Boundary rows in their own buffer (results in host memory): their
      // columns outside the part are final after the SSSP, so they cross the
      // host link now, while the FW runs; the decode then writes the part's
      // own columns straight into the result rows, after this copy.
      FAP_CUDA(cudaEventRecord(e->ev_copy[0], st));
      FAP_CUDA(cudaStreamWaitEvent(e->copy, e->ev_copy[0], 0));
      for (const auto &c : G.bnd_copies) {
        FAP_CUDA(cudaMemcpyAsync(static_cast<char *>(pl.dist) + c[0] * 4,
                                 static_cast<const char *>(pl.bdist) + c[1] * 4, (size_t)c[2] * 4,
                                 cudaMemcpyDefault, e->copy));
        if (pred)
          FAP_CUDA(cudaMemcpyAsync(reinterpret_cast<char *>(pl.pred) + c[0] * 4,
                                   reinterpret_cast<const char *>(pl.bpred) + c[1] * 4,
                                   (size_t)c[2] * 4, cudaMemcpyDefault, e->copy));
      }
      FAP_CUDA(cudaEventRecord(e->ev_copy[1], e->copy));
    }
    if (last) FAP_CUDA(rec(2));
    const int rounds = (int)G.diag.size();
    for (int r = 0; r < rounds; r++) {
      if (packed) {
        // Lookahead.  Pivot step r (one launch: round r - 1's update of block
        // row and column r, the closure, both panels) runs on the issuing
        // stream; round r's remaining tiles other than block row and column
        // r + 1 (`rest2`) on the side stream, where they overlap pivot step
        // r + 1.  Pivot step r waits for `rest2` of round r - 2 (the last
        // launch that wrote block row and column r); `rest2` of round r waits
        // for pivot step r.  Pivot step r + 1 and `rest2` of round r touch
        // disjoint entries: the pivot step reads block rows and columns r and
        // r + 1 and writes r + 1; `rest2` reads block row and column r outside
        // blocks r and r + 1 and writes neither.
        if (r >= 2) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1 + r % 2], 0));
        FAP_CUDA(fapk::launch_fw_pivot(pred, G.diag[r], G.diag_cnt[r], st));
        FAP_CUDA(cudaEventRecord(e->ev_fw[0], st));
        FAP_CUDA(cudaStreamWaitEvent(e->side, e->ev_fw[0], 0));
        FAP_CUDA(fapk::launch_fw_strips(pred, G.rest2[r], G.rest2_nseg[r], G.rest2_strips[r], e->side, false,
                                        G.tmaps));
        FAP_CUDA(cudaEventRecord(e->ev_fw[1 + r % 2], e->side));
      } else if (f32) {
        // FP32 lookahead, in strip launches: the pivot chain of round r
        // (round r - 1's update of block row and column r, the closure of
        // pivot block r, both panels) on the issuing stream, round r's
        // remaining tiles other than block row and column r + 1 (`rest2`) on
        // the side stream, beside the pivot chain of round r + 1.  The events
        // and the entries each side touches are those of the packed form.
        if (r >= 2) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1 + r % 2], 0));
        if (G.look_nseg[r] > 0)
          FAP_CUDA(fapk::launch_fw_strips(pred, G.look[r], G.look_nseg[r], G.look_strips[r], st, true, G.tmaps));
        FAP_CUDA(fapk::launch_fw_diag(f32, pred, G.diag[r], G.diag_cnt[r], st));
        if (G.pstrips_nseg[r] > 0)
          FAP_CUDA(fapk::launch_fw_strips(pred, G.pstrips[r], G.pstrips_nseg[r], G.pstrips_strips[r], st, true,
                                          G.tmaps));
        FAP_CUDA(cudaEventRecord(e->ev_fw[0], st));
        FAP_CUDA(cudaStreamWaitEvent(e->side, e->ev_fw[0], 0));
        if (G.rest2_nseg[r] > 0)
          FAP_CUDA(fapk::launch_fw_strips(pred, G.rest2[r], G.rest2_nseg[r], G.rest2_strips[r], e->side, true,
                                          G.tmaps));
        FAP_CUDA(cudaEventRecord(e->ev_fw[1 + r % 2], e->side));
      } else {
        FAP_CUDA(fapk::launch_fw_diag(f32, pred, G.diag[r], G.diag_cnt[r], st));
        {
          FAP_CUDA(fapk::launch_minplus_tiles(f32, pred, G.panel[r], G.panel_nseg[r], G.panel_tiles[r], packed, st));
          FAP_CUDA(fapk::launch_minplus_tiles(f32, pred, G.rest[r], G.rest_nseg[r], G.rest_tiles[r], packed, st));
        }
      }
    }
    if ((packed || f32) && rounds > 0) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1 + (rounds - 1) % 2], 0));  // join
    if (last) FAP_CUDA(rec(3));
    // Host results: the decode (own-part columns of the boundary rows, written
    // straight into the host rows) runs on the copy stream beside the
    // min-plus, after the FW and after the boundary rows' copy-out; the
    // min-plus reads neither those rows nor anything the decode writes.
    const bool decode_aside = !G.bnd_copies.empty();
    if (decode_aside) {
      FAP_CUDA(cudaEventRecord(e->ev_copy[0], st));
      FAP_CUDA(cudaStreamWaitEvent(e->copy, e->ev_copy[0], 0));
      FAP_CUDA(fapk::launch_decode(f32, pred, ba, pl.dist, pl.pred, e->copy));
      FAP_CUDA(cudaEventRecord(e->ev_copy[1], e->copy));
    }
    if (packed || f32) {  // strip form for the segments with K <= 100, tiles for the rest
      // The first class on the issuing stream, the later ones (a few parts
      // with larger K) on the low-priority side stream, whose CTAs take the
      // SMs the first launch leaves as it drains.  They write other parts'
      // rows and read only the FW matrices and the boundary rows.
      bool fork = false;
      for (int c = 1; c < G.mp_ncls; c++) fork = fork || (G.mp_cls_strips[c] > 0 && G.mp_cls_strips[0] > 0);
      if (fork) {
        FAP_CUDA(cudaEventRecord(e->ev_fw[0], st));
        FAP_CUDA(cudaStreamWaitEvent(e->side, e->ev_fw[0], 0));
      }
      for (int c = 0; c < G.mp_ncls; c++)
        FAP_CUDA(fapk::launch_minplus_strips(pred, G.mp + G.mp_cls_first[c], G.mp_cls_nseg[c],
                                             G.mp_cls_strips[c], G.mp_cls_max_k[c],
                                             fork && c > 0 ? e->side : st, f32,
                                             e->tile_cols ? e->tile_cols : G.mp_cls_cols[c], G.mp_aligned));
      FAP_CUDA(fapk::launch_minplus_tiles(f32, pred, G.mp, G.mp_nseg, G.mp_tiles - G.mp_strip_tiles,
                                          packed, st, G.mp_strip_tiles));
      if (fork) {  // join
        FAP_CUDA(cudaEventRecord(e->ev_fw[1], e->side));
        FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1], 0));
      }
    } else {
      FAP_CUDA(fapk::launch_minplus_tiles(f32, pred, G.mp, G.mp_nseg, G.mp_tiles, packed, st));
    }
    if (last) FAP_CUDA(rec(4));
    if (decode_aside) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_copy[1], 0));  // join
    else FAP_CUDA(fapk::launch_decode(f32, pred, ba, pl.dist, pl.pred, st));
    if (last) FAP_CUDA(rec(5));
    return FAP_OK;
  }
  // Host results: group g's finished rows go to the host rows on the copy
  // stream, behind the group's last launch; the issuing stream goes on with
  // the next group.  join() makes the issuing stream wait for every copy.
  int copy_out(size_t g) {
    if (!pl.hdist) return FAP_OK;
    const Plan::Group &G = pl.groups[g];
    FAP_CUDA(cudaEventRecord(e->ev_copy[0], st));
    FAP_CUDA(cudaStreamWaitEvent(e->copy, e->ev_copy[0], 0));
    const size_t off = (size_t)G.out_lo * 4, doff = (size_t)G.dev_lo * 4, bytes = (size_t)G.out_elems * 4;
    FAP_CUDA(cudaMemcpyAsync(static_cast<char *>(pl.hdist) + off, static_cast<const char *>(pl.dist) + doff,
                             bytes, cudaMemcpyDeviceToHost, e->copy));
    if (pl.hpred)
      FAP_CUDA(cudaMemcpyAsync(reinterpret_cast<char *>(pl.hpred) + off,
                               reinterpret_cast<const char *>(pl.pred) + doff, bytes,
                               cudaMemcpyDeviceToHost, e->copy));
    if (pl.ring_elems > 0) FAP_CUDA(cudaEventRecord(e->ev_slot[g & 1], e->copy));  // the slot is free again
    return FAP_OK;
  }
  // Two-slot staging: group g's first launch waits until the copy-out of
  // group g - 2 (the slot's previous rows) has finished.
  int slot_free(size_t g) {
    if (pl.ring_elems > 0 && g >= 2) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_slot[g & 1], 0));
    return FAP_OK;
  }
  int join() {
    if (!pl.hdist) return FAP_OK;
    FAP_CUDA(cudaEventRecord(e->ev_copy[1], e->copy));
    FAP_CUDA(cudaStreamWaitEvent(st, e->ev_copy[1], 0));
    return FAP_OK;
  }
  // Plain plans interleave per part (SSSP, rest); batched plans have one
  // group, or a few when the results go to host rows.
  int all() {
    int rc;
    const int c0 = fapk::launch_count();
    FAP_CUDA(rec(0));
    for (size_t g = 0; g < pl.groups.size(); g++) {
      if ((rc = slot_free(g)) != FAP_OK) return rc;
      if ((rc = sssp(g)) != FAP_OK) return rc;
      if (g + 1 == pl.groups.size()) FAP_CUDA(rec(1));
      if ((rc = rest(g, g + 1 == pl.groups.size())) != FAP_OK) return rc;
      if ((rc = copy_out(g)) != FAP_OK) return rc;
    }
    if ((rc = join()) != FAP_OK) return rc;
    pl.launches = fapk::launch_count() - c0;
    return FAP_OK;
  }
};

int check_status(fap_engine *e);
std::vector<const void *> buffer_signature(const fap_engine *e);

// SSSP autotuner: times the plan's SSSP phase (every group) with a few
// near-far steps -- multiples of the mean edge weight from 4 to 128, and
// plain frontier Bellman-Ford -- and keeps the fastest; then, when the plan
// carries batches of the other width (16 sources, two lane groups a warp, or
// 32, one), times both widths at that step (best of two runs each) and keeps
// the faster.  Step and width only order the work, so every candidate
// produces the same rows.  Runs once per engine, on the first run of a plan,
// when the step was left automatic; later plans take the chosen step and width.
int autotune_sssp(fap_engine *e, Plan &pl, cudaStream_t st) {
  const double unit = e->f32() ? e->wmean : std::max(1.0, e->wmean);
  const double factors[] = {4.0, 8.0, 16.0, 24.0, 32.0, 48.0, 64.0, 128.0, 0.0};
  double best = 0, best_ms = 1e300;
  cudaEvent_t a, b;
  FAP_CUDA(cudaEventCreate(&a));
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return set_error(FAP_ERR_CUDA, "autotune: event failed");
  }
  int rc = FAP_OK;
  auto time_phase = [&](double d, float &ms) {  // the SSSP phase at step d
    e->delta_try = d;
    Issuer is{e, pl, st, false};
    if (cudaEventRecord(a, st) != cudaSuccess) return set_error(FAP_ERR_CUDA, "autotune: event failed");
    for (size_t g = 0; g < pl.groups.size(); g++) {
      int r = is.sssp(g);
      if (r != FAP_OK) return r;
    }
    if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
        cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
      return set_error(FAP_ERR_CUDA, "autotune: event failed");
    return FAP_OK;
  };
  for (double f : factors) {
    double d = f > 0 ? f * unit : fapk::kSsspNoDelta;
    if (!e->f32()) d = std::max(1.0, std::floor(d));
    float ms = 0;
    if ((rc = time_phase(d, ms)) != FAP_OK) break;
    if (ms < best_ms) {
      best_ms = ms;
      best = d;
    }
  }
  if (rc == FAP_OK && pl.sssp_lanes_alt > 0) {
    auto swap_width = [&]() {
      std::swap(pl.sssp_lanes, pl.sssp_lanes_alt);
      for (auto &G : pl.groups) {
        std::swap(G.batches, G.batches_alt);
        std::swap(G.nbatches, G.nbatches_alt);
      }
    };
    float t[2] = {1e30f, 1e30f};  // [this width, the other]
    for (int w = 0; w < 2 && rc == FAP_OK; w++) {
      if (w == 1) swap_width();
      for (int rep = 0; rep < 2 && rc == FAP_OK; rep++) {
        float ms = 0;
        if ((rc = time_phase(best, ms)) == FAP_OK) t[w] = std::min(t[w], ms);
      }
    }
    if (rc == FAP_OK && t[1] >= t[0]) swap_width();  // back to the first width
    best_ms = std::min(t[0], t[1]);
    e->sssp_lanes_tuned = pl.sssp_lanes;
  }
  e->delta_try = 0;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != FAP_OK) return rc;
  if ((rc = check_status(e)) != FAP_OK) return rc;
  e->sssp_delta = best;
  e->tuned_ms = best_ms;
  pl.sig = buffer_signature(e);
  return FAP_OK;
}

// Automatic SSSP method: on the first run of a plan that can use the
// boundary graph, times the plan's SSSP phase (every group) through the
// boundary graph (a warm-up run, then the better of two) and as the
// whole-graph search at the current near-far step (once: it only has to lose
// clearly or win), keeps the faster for this plan and the engine's later
// plans, and reports it through fap_get_option.  Both methods give the same
// rows, so the trial runs rewrite the same boundary rows.
int trial_sssp_method(fap_engine *e, Plan &pl, cudaStream_t st) {
  cudaEvent_t a, b;
  FAP_CUDA(cudaEventCreate(&a));
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return set_error(FAP_ERR_CUDA, "method trial: event failed");
  }
  auto time_phase = [&](float &ms) {
    Issuer is{e, pl, st, false};
    if (cudaEventRecord(a, st) != cudaSuccess) return set_error(FAP_ERR_CUDA, "method trial: event failed");
    for (size_t g = 0; g < pl.groups.size(); g++) {
      int r = is.sssp(g);
      if (r != FAP_OK) return r;
    }
    if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
        cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
      return set_error(FAP_ERR_CUDA, "method trial: event failed");
    return FAP_OK;
  };
  int rc = FAP_OK;
  float tb = 1e30f, ts = 1e30f;
  pl.bsssp = 1;
  for (int rep = 0; rep < 3 && rc == FAP_OK; rep++) {
    float ms = 0;
    if ((rc = time_phase(ms)) == FAP_OK && rep > 0) tb = std::min(tb, ms);
  }
  if (rc == FAP_OK) {
    pl.bsssp = 0;
    rc = time_phase(ts);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  pl.bsssp = ts < tb ? 0 : 1;
  pl.method_trial = false;
  if (rc != FAP_OK) return rc;
  if ((rc = check_status(e)) != FAP_OK) return rc;
  e->sssp_method_tuned = pl.bsssp ? 2 : 1;
  pl.sig = buffer_signature(e);
  return FAP_OK;
}

// Tile autotuner of the packed min-plus (strip form): on a plan's first run,
// once the product's inputs are in place (closed FW matrices, boundary
// rows), times every strip class launch of every group with 128 x 64 and
// 128 x 128 tiles (best of two launches each) and keeps the faster for the
// plan's later runs and its CUDA graph.  The product is a pure function of
// those inputs -- the part's own columns come from its FW matrix, every
// other output from the product, whatever the output held -- so the trial
// launches rewrite the same rows.  Not run for results in mapped host
// memory, where the host link bounds every tile width.
int autotune_tiles(fap_engine *e, Plan &pl, cudaStream_t st) {
  if (pl.pack != 1 || pl.bdist != nullptr) return FAP_OK;
  const bool pred = pl.pred != nullptr;
  cudaEvent_t a, b;
  FAP_CUDA(cudaEventCreate(&a));
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return set_error(FAP_ERR_CUDA, "autotune: event failed");
  }
  int rc = FAP_OK;
  for (auto &G : pl.groups) {
    for (int c = 0; c < G.mp_ncls && rc == FAP_OK; c++) {
      if (G.mp_cls_strips[c] <= 0) continue;
      float best_ms = 1e30f;
      int best = 0;
      for (int cols : {64, 128}) {
        float t = 1e30f;
        for (int rep = 0; rep < 2 && rc == FAP_OK; rep++) {
          cudaError_t ce = cudaEventRecord(a, st);
          if (ce == cudaSuccess)
            ce = fapk::launch_minplus_strips(pred, G.mp + G.mp_cls_first[c], G.mp_cls_nseg[c],
                                             G.mp_cls_strips[c], G.mp_cls_max_k[c], st, false, cols,
                                             G.mp_aligned);
          if (ce == cudaSuccess) ce = cudaEventRecord(b, st);
          if (ce == cudaSuccess) ce = cudaEventSynchronize(b);
          float ms = 0;
          if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, a, b);
          if (ce != cudaSuccess) {
            rc = set_error(FAP_ERR_CUDA, std::string("tile autotune: ") + cudaGetErrorString(ce));
            break;
          }
          t = std::min(t, ms);
        }
        if (rc == FAP_OK && t < best_ms) {
          best_ms = t;
          best = cols;
        }
      }
      G.mp_cls_cols[c] = best;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != FAP_OK) return rc;
  return check_status(e);
}

// Decides the packed int32 form for a plan on its first run: runs every
// group's SSSP, reads back the largest finite SSSP distance, and checks the
// bound of every finite result: a path inside a part to its first boundary
// vertex ((max part size - 1) * max weight) plus an SSSP distance from that
// boundary vertex.  Afterwards runs the rest of every group.
int first_run(fap_engine *e, Plan &pl, cudaStream_t st) {
  Issuer is{e, pl, st, false};
  int rc;
  if (e->f32()) {
    pl.pack = 0;
    return is.all();
  }
  FAP_CUDA(cudaMemsetAsync(e->d_status + 1, 0, sizeof(unsigned), st));
  FAP_CUDA(is.rec(0));
  for (size_t g = 0; g < pl.groups.size(); g++)
    if ((rc = is.sssp(g)) != FAP_OK) return rc;
  FAP_CUDA(is.rec(1));
  unsigned maxd = 0;
  FAP_CUDA(cudaMemcpyAsync(&maxd, e->d_status + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  FAP_CUDA(cudaStreamSynchronize(st));
  const unsigned long long bound =
      (unsigned long long)maxd + (unsigned long long)std::max(pl.max_sub - 1, 0) * e->wmax;
  const bool k_ok = pl.pred == nullptr || pl.max_mp_k <= fapk::max_packed_k();
  pl.pack = (e->int32_form == 0 && bound < fapk::pack_limit() && k_ok) ? 1 : 0;
  for (size_t g = 0; g < pl.groups.size(); g++) {
    if ((rc = is.rest(g, g + 1 == pl.groups.size())) != FAP_OK) return rc;
    if ((rc = is.copy_out(g)) != FAP_OK) return rc;
  }
  return is.join();
}

int check_status(fap_engine *e) {
  unsigned h = 0;
  FAP_CUDA(cudaMemcpy(&h, e->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (h) {
    FAP_CUDA(cudaMemset(e->d_status, 0, sizeof(unsigned)));
    if (h & fapk::kErrSsspCap) return set_error(FAP_ERR_NOT_CONVERGED, "SSSP reached its iteration cap");
    return set_error(FAP_ERR_INVALID, "a kernel saw an out-of-range index");
  }
  unsigned t = 0;
  FAP_CUDA(fapk::tma_status(&t, true));
  if (t) return set_error(FAP_ERR_CUDA, "a bulk tensor copy of the Floyd-Warshall tiles did not complete");
  return FAP_OK;
}

std::vector<const void *> buffer_signature(const fap_engine *e) {
  double d = sssp_delta_of(e);
  intptr_t dbits;
  std::memcpy(&dbits, &d, sizeof(dbits));
  return {e->fw_d.p, e->fw_p.p, e->sssp_scratch.p, e->sssp_bits.p,
          reinterpret_cast<const void *>((intptr_t)e->sssp_slots_alloc),
          reinterpret_cast<const void *>((intptr_t)e->sssp_fp64),
          reinterpret_cast<const void *>((intptr_t)e->sssp_lanes),
          reinterpret_cast<const void *>((intptr_t)e->tile_cols),
          reinterpret_cast<const void *>((intptr_t)e->sssp_method),
          reinterpret_cast<const void *>((intptr_t)e->int32_form),
          e->bg_tab.p,
          reinterpret_cast<const void *>(dbits),
          reinterpret_cast<const void *>((intptr_t)std::llround(e->host_group_mb * 1024.0))};
}

Plan *find_plan(fap_engine *e, int mode, void *dist, int32_t *pred,
                const std::vector<int32_t> &parts, const std::vector<int64_t> &offs, void *bdist,
                int32_t *bpred, void *hdist, int32_t *hpred, int64_t ring_elems) {
  const std::vector<const void *> sig = buffer_signature(e);
  for (auto &p : e->plans)
    if (p->mode == mode && p->dist == dist && p->pred == pred && p->parts == parts &&
        p->row_offs == offs && p->bdist == bdist && p->bpred == bpred && p->hdist == hdist &&
        p->ring_elems == ring_elems &&
        p->hpred == hpred && p->sig == sig)
      return p.get();
  return nullptr;
}

// Runs `parts` (row offsets `offs` into dist/pred, device-accessible).  With
// bdist, the parts' boundary rows go to that device buffer instead (part i's
// at element boffs[i]) and dist/pred receive only the inner rows.
int run_parts(fap_engine *e, int mode, void *dist, int32_t *pred, const std::vector<int32_t> &parts,
              const std::vector<int64_t> &offs, cudaStream_t st, void *bdist = nullptr,
              int32_t *bpred = nullptr, const std::vector<int64_t> &boffs = {}, void *hdist = nullptr,
              int32_t *hpred = nullptr, int64_t ring_elems = 0) {
  int rc;
  // work buffers
  size_t fw_elems = 0;
  int64_t batches8 = 0, batches32 = 0;
  for (int p : parts) {
    size_t ld = align_up((size_t)e->ver_num[p], (size_t)fapk::fw_block());
    fw_elems += ld * ld;
    batches8 += (e->bdy_num[p] + 7) / 8;
    batches32 += (e->bdy_num[p] + 31) / 32;
  }
  const bool acc64 = e->f32() && e->sssp_fp64;
  int lanes = e->sssp_lanes                        ? e->sssp_lanes
              : (e->sssp_lanes_tuned && !acc64) ? e->sssp_lanes_tuned
                                                : fapk::sssp_lanes_for(batches8, batches32, e->sm_count, acc64);
  if (acc64 && lanes == 8) lanes = 16;  // the FP64 search has no 8-source form
  // Boundary SSSP through the boundary graph where its arithmetic is exact
  // (int32 graphs; FP32 graphs with the FP64 option and a fixed-point
  // shift), its shared-memory tables fit and every batch of a group gets a
  // table slot of its own; otherwise the whole-graph search.
  bool bs = false, trial = false;
  if (e->sssp_method != 1 && e->sssp_method_tuned != 1 && (!e->f32() || acc64)) {
    if ((rc = prepare_bgraph(e)) != FAP_OK) return rc;
    if (e->bg_ok) {
      int64_t nb = 0;
      for (int p : parts) nb += (e->bdy_num[p] + lanes - 1) / lanes;
      bs = nb <= max_sssp_slots(e, acc64 && lanes == 32);
    }
    // automatic: the first run times both methods (the search wins where few
    // vertices are reachable from the boundary, as on sparse directed graphs)
    trial = bs && e->sssp_method == 0 && e->sssp_method_tuned == 0 && e->autotune;
  }
  // The SSSP autotuner also tries a second batch width (8 -> 16, 16 -> 32,
  // 32 -> 16; not for the FP64 search, whose 32-source slots have another
  // layout); scratch for the larger batch count of the two.
  const bool tune_lanes = e->autotune && e->sssp_delta <= 0 && e->sssp_lanes == 0 && !acc64 && !bs;
  const int alt_lanes = lanes == 16 ? 32 : 16;
  const bool wide = acc64 && lanes == 32;
  const int count_lanes = tune_lanes ? std::min(lanes, alt_lanes) : lanes;
  int max_batches = 0;
  for (int p : parts) max_batches += (e->bdy_num[p] + count_lanes - 1) / count_lanes;
  if ((rc = e->fw_d.ensure(std::max<size_t>(fw_elems, 1) * 4)) != FAP_OK) return rc;
  if (pred && (rc = e->fw_p.ensure(std::max<size_t>(fw_elems, 1) * 4)) != FAP_OK) return rc;
  int slots = std::min(std::max(max_batches, 1), max_sssp_slots(e, wide));
  if ((rc = ensure_sssp_scratch(e, slots, wide)) != FAP_OK) return rc;

  Plan *pl = find_plan(e, mode, dist, pred, parts, offs, bdist, bpred, hdist, hpred, ring_elems);
  if (!pl) {
    if (e->plans.size() >= 8) e->plans.erase(e->plans.begin());
    auto np = std::make_unique<Plan>();
    np->mode = mode;
    np->dist = dist;
    np->pred = pred;
    np->parts = parts;
    np->row_offs = offs;
    np->bdist = bdist;
    np->bpred = bpred;
    np->brow_offs = boffs;
    np->hdist = hdist;
    np->hpred = hpred;
    np->ring_elems = ring_elems;
    np->sig = buffer_signature(e);
    np->sssp_lanes = lanes;
    np->sssp_lanes_alt = tune_lanes ? alt_lanes : 0;
    np->bsssp = bs ? 1 : 0;
    np->method_trial = trial;
    if ((rc = build_plan(e, *np)) != FAP_OK) return rc;
    e->plans.push_back(std::move(np));
    pl = e->plans.back().get();
  }
  if (pl->pack < 0) {  // first run: trials and tuners, then the plan without a graph
    const int c0 = fapk::launch_count();
    if (pl->method_trial && (rc = trial_sssp_method(e, *pl, st)) != FAP_OK) return rc;
    if (e->autotune && e->sssp_delta <= 0 && !pl->bsssp && (rc = autotune_sssp(e, *pl, st)) != FAP_OK)
      return rc;
    if ((rc = first_run(e, *pl, st)) != FAP_OK) return rc;
    e->fw_host_work += pl->pack == 1 ? pl->fw_pivot_work : pl->fw_tile_work;
    if (e->autotune && e->tile_cols == 0 && (rc = autotune_tiles(e, *pl, st)) != FAP_OK) return rc;
    e->last_launches = fapk::launch_count() - c0;  // every kernel of this call, trials included
    return FAP_OK;
  }
  if (mode == FAP_MODE_BATCHED) {
    if (!pl->exec) {
      cudaGraph_t graph = nullptr;
      cudaStream_t cap = e->stream;
      FAP_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      Issuer is{e, *pl, cap, true};
      int irc = is.all();
      cudaError_t ce = cudaStreamEndCapture(cap, &graph);
      if (irc != FAP_OK) {
        if (graph) cudaGraphDestroy(graph);
        return irc;
      }
      if (ce != cudaSuccess) return set_error(FAP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      // kernel nodes keep the priority of the stream they were captured from
      ce = cudaGraphInstantiate(&pl->exec, graph, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        pl->exec = nullptr;
        return set_error(FAP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
      }
    }
    if (st != e->stream) {
      FAP_CUDA(cudaEventRecord(e->ev_sync[0], st));
      FAP_CUDA(cudaStreamWaitEvent(e->stream, e->ev_sync[0], 0));
    }
    FAP_CUDA(cudaGraphLaunch(pl->exec, e->stream));
    if (st != e->stream) {
      FAP_CUDA(cudaEventRecord(e->ev_sync[1], e->stream));
      FAP_CUDA(cudaStreamWaitEvent(st, e->ev_sync[1], 0));
    }
  } else {
    Issuer is{e, *pl, st, false};
    if ((rc = is.all()) != FAP_OK) return rc;
  }
  e->fw_host_work += pl->pack == 1 ? pl->fw_pivot_work : pl->fw_tile_work;
  e->last_launches = pl->launches;
  return FAP_OK;
}

void read_times(fap_engine *e) {
  float t[5] = {0, 0, 0, 0, 0};
  cudaEventElapsedTime(&t[0], e->ev[0], e->ev[1]);  // sssp
  float b = 0, f = 0, mp = 0, dc = 0;
  cudaEventElapsedTime(&b, e->ev[1], e->ev[2]);
  cudaEventElapsedTime(&f, e->ev[2], e->ev[3]);
  cudaEventElapsedTime(&mp, e->ev[3], e->ev[4]);
  cudaEventElapsedTime(&dc, e->ev[4], e->ev[5]);
  float tot = 0;
  cudaEventElapsedTime(&tot, e->ev[0], e->ev[5]);
  (void)cudaGetLastError();
  e->times[0] = t[0];
  e->times[1] = f;
  e->times[2] = mp;
  e->times[3] = b + dc;
  e->times[4] = tot;
}

cudaStream_t pick_stream(fap_engine *e, void *stream) {
  return stream ? static_cast<cudaStream_t>(stream) : e->stream;
}

int init_device(fap_engine *e, int device) {
  int count = 0;
  cudaError_t ce = cudaGetDeviceCount(&count);
  if (ce != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    return set_error(FAP_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= count) return set_error(FAP_ERR_INVALID, "device ordinal out of range");
  FAP_CUDA(cudaSetDevice(device));
  // two attributes, not cudaGetDeviceProperties (which queries every property
  // and costs milliseconds per engine)
  int major = 0, sms = 0;
  FAP_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
  FAP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  if (major < 10) return set_error(FAP_ERR_NO_DEVICE, "the engine is built for sm_103a (Blackwell Ultra) only");
  e->device = device;
  e->sm_count = sms;
  int prio_low = 0, prio_high = 0;
  FAP_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  FAP_CUDA(cudaStreamCreateWithPriority(&e->stream, cudaStreamNonBlocking, prio_high));
  FAP_CUDA(cudaStreamCreateWithPriority(&e->side, cudaStreamNonBlocking, prio_low));
  for (auto &ev : e->ev) FAP_CUDA(cudaEventCreate(&ev));
  for (auto &ev : e->ev_sync) FAP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  for (auto &ev : e->ev_fw) FAP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  FAP_CUDA(cudaStreamCreateWithFlags(&e->copy, cudaStreamNonBlocking));
  for (auto &ev : e->ev_copy) FAP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  for (auto &ev : e->ev_slot) FAP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  // status words: [0] error flags, [1]/[2] maxima for the packed-form bound
  FAP_CUDA(cudaMalloc(&e->d_status, 4 * sizeof(unsigned)));
  FAP_CUDA(cudaMemset(e->d_status, 0, 4 * sizeof(unsigned)));
  FAP_CUDA(cudaMalloc(&e->d_stats, 8 * sizeof(unsigned long long)));
  FAP_CUDA(cudaMemset(e->d_stats, 0, 8 * sizeof(unsigned long long)));
  FAP_CUDA(fapk::init_minplus_kernels());
  FAP_CUDA(fapk::init_sssp_kernels());
  FAP_CUDA(fapk::init_bg_kernels());
  return FAP_OK;
}

// Shift s such that every weight is an integer multiple of 2^-s and every
// simple path stays below 2^52 such units ((n - 1) * max weight * 2^s <
// 2^52): then path lengths are exact in 64-bit fixed point and in FP64
// (sums of multiples of 2^-s below 2^(52 - s)).  -1 when there is none.
int fixed_point_shift(const float *w, int64_t m, int32_t n, float wmax) {
  int s = 0;
  for (int64_t j = 0; j < m; j++) {
    if (!(w[j] > 0.0f)) continue;
    int ex = 0;
    const float f = std::frexp(w[j], &ex);  // w = f * 2^ex, f in [0.5, 1)
    uint32_t mant = (uint32_t)std::ldexp(f, 24);  // exact: at most 24 significant bits
    int low = ex - 24;
    while (!(mant & 1u)) {
      mant >>= 1;
      low++;
    }
    s = std::max(s, -low);  // w = mant * 2^low
  }
  if (s > 200) return -1;
  const double bound = std::ldexp((double)wmax * (double)std::max<int32_t>(n - 1, 1), s);
  return bound < std::ldexp(1.0, 52) ? s : -1;
}

template <typename T>
int upload(T **dst, const T *src, size_t count) {
  FAP_CUDA(cudaMalloc((void **)dst, std::max<size_t>(count, 1) * sizeof(T)));
  if (count) FAP_CUDA(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return FAP_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace

// ============================ C ABI ========================================
extern "C" {

const char *fap_version(void) { return "fastapsp-gb300 0.1 (sm_103a)"; }

const char *fap_status_string(int status) {
  switch (status) {
    case FAP_OK: return "ok";
    case FAP_ERR_INVALID: return "invalid argument";
    case FAP_ERR_CUDA: return "CUDA error";
    case FAP_ERR_NOMEM: return "out of memory";
    case FAP_ERR_STATE: return "invalid state";
    case FAP_ERR_NOT_CONVERGED: return "SSSP did not converge";
    case FAP_ERR_IO: return "I/O error";
    case FAP_ERR_NO_DEVICE: return "no suitable CUDA device";
    case FAP_ERR_RANGE: return "value out of range";
    default: return "unknown status";
  }
}

const char *fap_last_error(void) { return fapi::last_error(); }

int fap_device_count(int32_t *count) {
  if (!count) return set_error(FAP_ERR_INVALID, "null count");
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) {
    (void)cudaGetLastError();
    c = 0;
  }
  *count = c;
  return FAP_OK;
}

int fap_mtx_counts(const char *path, int32_t directed, int32_t weighted, int32_t *n, int64_t *m) {
  (void)weighted;
  if (!path || !n || !m) return set_error(FAP_ERR_INVALID, "null argument");
  return fapi::mtx_counts(path, directed != 0, n, m);
}

int fap_mtx_read(const char *path, int32_t directed, int32_t weighted, int32_t n, int64_t m,
                 int32_t *adj_size, int32_t *row_offset, int32_t *col_val, float *weight) {
  if (!path || !adj_size || !row_offset || (m > 0 && (!col_val || !weight)))
    return set_error(FAP_ERR_INVALID, "null argument");
  return fapi::mtx_read(path, directed != 0, weighted != 0, n, m, adj_size, row_offset, col_val,
                        weight);
}

int fap_partition(int32_t n, const int32_t *row_offset, const int32_t *col_val, int32_t K,
                  uint64_t seed, int32_t *graph_id, int64_t *edge_cut) {
  if (!row_offset || !graph_id || (n > 0 && !col_val && row_offset[n] > 0))
    return set_error(FAP_ERR_INVALID, "null argument");
  return fapi::partition(n, row_offset, col_val, K, seed, graph_id, edge_cut);
}

int fap_preprocess(int32_t K, int32_t n, const int32_t *graph_id, const int32_t *row_offset,
                   const int32_t *col_val, int32_t *st2ed, int32_t *ed2st, int32_t *ver_num,
                   int32_t *ver_offset, int32_t *bdy_num, int32_t *bdy_offset) {
  if (!graph_id || !row_offset || !st2ed || !ed2st || !ver_num || !ver_offset || !bdy_num ||
      !bdy_offset)
    return set_error(FAP_ERR_INVALID, "null argument");
  return fapi::preprocess(K, n, graph_id, row_offset, col_val, st2ed, ed2st, ver_num, ver_offset,
                          bdy_num, bdy_offset, nullptr);
}

int fap_create_context(int32_t device, fap_engine **out) {
  if (!out) return set_error(FAP_ERR_INVALID, "null out");
  *out = nullptr;
  auto e = std::make_unique<fap_engine>();
  int rc = init_device(e.get(), device);
  if (rc != FAP_OK) {
    fap_destroy(e.release());
    return rc;
  }
  *out = e.release();
  return FAP_OK;
}

int fap_create(int32_t n, int64_t m, const int32_t *row_offset, const int32_t *col_val,
               const float *weight, int32_t K, const int32_t *graph_id, int32_t dtype,
               int32_t device, fap_engine **out) {
  if (!out) return set_error(FAP_ERR_INVALID, "null out");
  *out = nullptr;
  if (n < 0 || m < 0 || K < 1 || !row_offset || (m > 0 && (!col_val || !weight)))
    return set_error(FAP_ERR_INVALID, "fap_create: bad graph arguments");
  if (dtype != FAP_DTYPE_F32 && dtype != FAP_DTYPE_I32)
    return set_error(FAP_ERR_INVALID, "fap_create: unknown dtype");
  if (row_offset[0] != 0 || (int64_t)row_offset[n] != m)
    return set_error(FAP_ERR_INVALID, "fap_create: row_offset must start at 0 and end at m");
  for (int32_t i = 0; i < n; i++)
    if (row_offset[i + 1] < row_offset[i]) return set_error(FAP_ERR_INVALID, "fap_create: row_offset not monotone");
  float wmax = 0.0f;
  for (int64_t j = 0; j < m; j++) {
    if (col_val[j] < 0 || col_val[j] >= n) return set_error(FAP_ERR_INVALID, "fap_create: column id out of range");
    float wj = weight[j];
    if (!(wj >= 0.0f) || std::isinf(wj)) return set_error(FAP_ERR_RANGE, "fap_create: weights must be finite and >= 0");
    if (dtype == FAP_DTYPE_I32 && wj != std::floor(wj))
      return set_error(FAP_ERR_RANGE, "fap_create: int32 mode needs integer weights");
    wmax = std::max(wmax, wj);
  }
  if (dtype == FAP_DTYPE_I32 && (double)wmax * std::max<int64_t>(n - 1, 1) >= (double)FAP_INF_I32)
    return set_error(FAP_ERR_RANGE, "fap_create: (n-1) * max weight must stay below 2^30 in int32 mode");

  auto e = std::make_unique<fap_engine>();
  e->n = n;
  e->m = m;
  e->K = K;
  e->dtype = dtype;
  e->ro.assign(row_offset, row_offset + n + 1);
  e->col.assign(col_val, col_val + m);
  e->w.assign(weight, weight + m);
  e->graph_id.resize(n);
  int rc;
  if (graph_id) {
    for (int32_t i = 0; i < n; i++) {
      if (graph_id[i] < 1 || graph_id[i] > K) return set_error(FAP_ERR_INVALID, "fap_create: part id outside 1..K");
      e->graph_id[i] = graph_id[i];
    }
  } else {
    if ((rc = fapi::partition(n, row_offset, col_val, K, 1, e->graph_id.data(), nullptr)) != FAP_OK) return rc;
  }
  e->st2ed.resize(n);
  e->ed2st.resize(n);
  e->ver_num.resize(K + 1);
  e->ver_offset.resize(K + 1);
  e->bdy_num.resize(K + 1);
  e->bdy_offset.resize(K + 1);
  if ((rc = fapi::preprocess(K, n, e->graph_id.data(), row_offset, col_val, e->st2ed.data(),
                             e->ed2st.data(), e->ver_num.data(), e->ver_offset.data(),
                             e->bdy_num.data(), e->bdy_offset.data(), nullptr)) != FAP_OK)
    return rc;
  if ((rc = init_device(e.get(), device)) != FAP_OK) {
    fap_destroy(e.release());
    return rc;
  }
  // in-edge CSR (counting sort by destination, sources ascending)
  std::vector<int32_t> iro(n + 1, 0), icol(m);
  std::vector<float> iw(m);
  for (int64_t j = 0; j < m; j++) iro[col_val[j] + 1]++;
  for (int32_t i = 0; i < n; i++) iro[i + 1] += iro[i];
  {
    std::vector<int32_t> fill(iro.begin(), iro.end() - 1);
    for (int32_t u = 0; u < n; u++)
      for (int32_t j = row_offset[u]; j < row_offset[u + 1]; j++) {
        int32_t pos = fill[col_val[j]]++;
        icol[pos] = u;
        iw[pos] = weight[j];
      }
  }
  std::vector<uint32_t> wbits(m), iwbits(m);
  for (int64_t j = 0; j < m; j++) {
    if (dtype == FAP_DTYPE_F32) {
      std::memcpy(&wbits[j], &weight[j], 4);
      std::memcpy(&iwbits[j], &iw[j], 4);
    } else {
      wbits[j] = (uint32_t)weight[j];
      iwbits[j] = (uint32_t)iw[j];
    }
  }
  fap_engine *E = e.get();
  if ((rc = upload(&E->d_ro, row_offset, (size_t)n + 1)) != FAP_OK ||
      (rc = upload(&E->d_col, col_val, (size_t)m)) != FAP_OK ||
      (rc = upload(&E->d_iro, iro.data(), (size_t)n + 1)) != FAP_OK ||
      (rc = upload(&E->d_icol, icol.data(), (size_t)m)) != FAP_OK ||
      (rc = upload(&E->d_gid, E->graph_id.data(), (size_t)n)) != FAP_OK ||
      (rc = upload(&E->d_st2ed, E->st2ed.data(), (size_t)n)) != FAP_OK ||
      (rc = upload(&E->d_ed2st, E->ed2st.data(), (size_t)n)) != FAP_OK ||
      (rc = upload((uint32_t **)&E->d_w, wbits.data(), (size_t)m)) != FAP_OK ||
      (rc = upload((uint32_t **)&E->d_iw, iwbits.data(), (size_t)m)) != FAP_OK) {
    fap_destroy(e.release());
    return rc;
  }
  E->wmax = dtype == FAP_DTYPE_I32 ? (uint32_t)wmax : 0u;
  if (dtype == FAP_DTYPE_F32) E->fix_shift = fixed_point_shift(weight, m, n, wmax);
  {
    double sum = 0;
    for (int64_t j = 0; j < m; j++) sum += weight[j];
    E->wmean = m > 0 ? std::max(sum / (double)m, 1e-30) : 1.0;
  }
  E->has_graph = true;
  *out = e.release();
  return FAP_OK;
}

int fap_destroy(fap_engine *e) {
  if (!e) return FAP_OK;
  {
    DeviceGuard g(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->plans.clear();
    e->fw_d.release();
    e->fw_p.release();
    e->sssp_scratch.release();
    e->sssp_bits.release();
    e->res_d.release();
    e->res_p.release();
    e->bnd_d.release();
    e->bnd_p.release();
    e->small.release();
    e->bg_tab.release();
    e->bg_L.release();
    e->bg_DS.release();
    void *ptrs[] = {e->d_ro, e->d_col, e->d_iro, e->d_icol, e->d_gid, e->d_st2ed, e->d_ed2st,
                    e->d_w, e->d_iw, e->d_status, e->d_stats};
    for (void *p : ptrs)
      if (p) cudaFree(p);
    for (auto &ev : e->ev)
      if (ev) cudaEventDestroy(ev);
    for (auto &ev : e->ev_sync)
      if (ev) cudaEventDestroy(ev);
    for (auto &ev : e->ev_fw)
      if (ev) cudaEventDestroy(ev);
    for (auto &ev : e->ev_copy)
      if (ev) cudaEventDestroy(ev);
    for (auto &ev : e->ev_slot)
      if (ev) cudaEventDestroy(ev);
    if (e->copy) cudaStreamDestroy(e->copy);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->side) cudaStreamDestroy(e->side);
    (void)cudaGetLastError();
  }
  delete e;
  return FAP_OK;
}

int fap_num_vertices(const fap_engine *e, int32_t *n, int32_t *K) {
  if (!e || !n || !K) return set_error(FAP_ERR_INVALID, "null argument");
  *n = e->n;
  *K = e->K;
  return FAP_OK;
}

int fap_mapping(const fap_engine *e, int32_t *st2ed) {
  if (!e || !st2ed) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  std::copy(e->st2ed.begin(), e->st2ed.end(), st2ed);
  return FAP_OK;
}

int fap_graph_id(const fap_engine *e, int32_t *graph_id) {
  if (!e || !graph_id) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  std::copy(e->graph_id.begin(), e->graph_id.end(), graph_id);
  return FAP_OK;
}

int fap_part_info(const fap_engine *e, int32_t part, int32_t *sub, int32_t *bdy, int32_t *offset) {
  if (!e) return set_error(FAP_ERR_INVALID, "null engine");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (part < 1 || part > e->K) return set_error(FAP_ERR_INVALID, "part id outside 1..K");
  if (sub) *sub = e->ver_num[part];
  if (bdy) *bdy = e->bdy_num[part];
  if (offset) *offset = e->ver_offset[part];
  return FAP_OK;
}

// Device address of page-locked, mapped host memory (null otherwise).
static void *mapped_host_ptr(void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

static int solve_common(fap_engine *e, const std::vector<int32_t> &parts, int64_t rows, void *dist,
                        int32_t *pred, int mode, void *stream) {
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  fapi::clear_error();
  cudaStream_t st = pick_stream(e, stream);
  const size_t bytes = (size_t)rows * e->n * 4;
  const bool dev_d = is_device_ptr(dist);
  const bool dev_p = pred == nullptr || is_device_ptr(pred);
  std::vector<int64_t> offs;
  int64_t acc = 0;
  for (int32_t p : parts) {
    offs.push_back(acc * e->n);
    acc += e->ver_num[p];
  }
  int rc;
  // Page-locked host results: the kernels write the inner rows straight into
  // them (no device copy of the n x n result, and the copy-out overlaps the
  // min-plus); the boundary rows, which the FW build and the min-plus read
  // back, stay in a device buffer, copied out right after the SSSP (during
  // the FW), and the decode then writes their own-part columns in place.
  void *hd = dev_d ? nullptr : mapped_host_ptr(dist);
  void *hp = (pred && !dev_p) ? mapped_host_ptr(pred) : nullptr;
  bool direct = !dev_d && hd && (pred == nullptr || hp);
  if (direct && e->host_results == 0) {
    // Staged instead when the device has room for a copy of the results:
    // kernel stores into host memory reached only ~45 GB/s on the
    // 114,599-vertex graph (rows 458 KB apart, every tile touching 128 of
    // them), while the copy engines move the finished rows at the host
    // link's rate.
    const size_t need = bytes * (pred && !dev_p ? 2 : 1);
    const size_t have = (e->res_d.bytes >= bytes ? bytes : 0) + (pred && e->res_p.bytes >= bytes ? bytes : 0);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      (void)cudaGetLastError();
      free_b = 0;
    }
    if (need <= have || need - have + ((size_t)2 << 30) <= free_b) direct = false;
  }
  if (direct) {
    std::vector<int64_t> boffs;
    int64_t bacc = 0;
    for (int32_t p : parts) {
      boffs.push_back(bacc * e->n);
      bacc += e->bdy_num[p];
    }
    const size_t bbytes = std::max<size_t>((size_t)bacc * e->n * 4, 4);
    if ((rc = e->bnd_d.ensure(bbytes)) != FAP_OK) return rc;
    if (pred && (rc = e->bnd_p.ensure(bbytes)) != FAP_OK) return rc;
    int32_t *bp = pred ? static_cast<int32_t *>(e->bnd_p.p) : nullptr;
    if ((rc = run_parts(e, mode, hd, static_cast<int32_t *>(hp), parts, offs, st, e->bnd_d.p, bp,
                        boffs)) != FAP_OK)
      return rc;
  } else {
    void *dd = dist;
    int32_t *dp = pred;
    // Page-locked host rows (both, when there are predecessors): the plan
    // copies each group's rows as it finishes; otherwise one copy at the end.
    const bool plan_copies = !dev_d && hd && (pred == nullptr || (!dev_p && hp));
    // With three or more groups (FP32, batched: every group runs start to
    // end before the next) the device copy is two group-sized slots that the
    // groups take in turn instead of all the rows: a quarter of the device
    // memory on the 114,599-vertex graph, and less to allocate and free.
    int64_t ring = 0;
    size_t dbytes = bytes;
    if (plan_copies && mode == FAP_MODE_BATCHED && e->f32()) {
      const std::vector<std::vector<int>> hg = host_groups(e, parts, pred != nullptr);
      if (hg.size() >= 3) {
        for (const auto &grp : hg) {
          int64_t rows = 0;
          for (int i : grp) rows += e->ver_num[parts[i]];
          ring = std::max(ring, rows * e->n);
        }
        dbytes = (size_t)ring * 2 * 4;
      }
    }
    if (!dev_d) {
      if ((rc = e->res_d.ensure(std::max<size_t>(dbytes, 4))) != FAP_OK) return rc;
      dd = e->res_d.p;
    }
    if (pred && !dev_p) {
      if ((rc = e->res_p.ensure(std::max<size_t>(dbytes, 4))) != FAP_OK) return rc;
      dp = static_cast<int32_t *>(e->res_p.p);
    }
    if (plan_copies) {
      if ((rc = run_parts(e, mode, dd, dp, parts, offs, st, nullptr, nullptr, {}, dist, pred, ring)) != FAP_OK)
        return rc;
    } else {
      if ((rc = run_parts(e, mode, dd, dp, parts, offs, st)) != FAP_OK) return rc;
      if (!dev_d) FAP_CUDA(cudaMemcpyAsync(dist, dd, bytes, cudaMemcpyDeviceToHost, st));
      if (pred && !dev_p) FAP_CUDA(cudaMemcpyAsync(pred, dp, bytes, cudaMemcpyDeviceToHost, st));
    }
  }
  FAP_CUDA(cudaStreamSynchronize(st));
  if (mode == FAP_MODE_BATCHED && st != e->stream) FAP_CUDA(cudaStreamSynchronize(e->stream));
  read_times(e);
  return check_status(e);
}

int fap_solve_part(fap_engine *e, int32_t part, void *dist, int32_t *pred, void *stream) {
  if (!e || !dist) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (part < 1 || part > e->K) return set_error(FAP_ERR_INVALID, "part id outside 1..K");
  return solve_common(e, {part}, e->ver_num[part], dist, pred, FAP_MODE_PLAIN, stream);
}

int fap_solve(fap_engine *e, void *dist, int32_t *pred, int32_t mode, void *stream) {
  if (!e || !dist) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (mode != FAP_MODE_PLAIN && mode != FAP_MODE_BATCHED) return set_error(FAP_ERR_INVALID, "unknown mode");
  std::vector<int32_t> parts;
  for (int32_t p = 1; p <= e->K; p++) parts.push_back(p);
  return solve_common(e, parts, e->n, dist, pred, mode, stream);
}

int fap_solve_parts(fap_engine *e, const int32_t *parts, int32_t nparts, void *dist, int32_t *pred,
                    int32_t mode, void *stream) {
  if (!e || !dist || !parts || nparts < 1) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (mode != FAP_MODE_PLAIN && mode != FAP_MODE_BATCHED) return set_error(FAP_ERR_INVALID, "unknown mode");
  std::vector<int32_t> list(parts, parts + nparts);
  std::vector<char> seen(e->K + 1, 0);
  int64_t rows = 0;
  for (int32_t p : list) {
    if (p < 1 || p > e->K) return set_error(FAP_ERR_INVALID, "part id outside 1..K");
    if (seen[p]++) return set_error(FAP_ERR_INVALID, "part listed twice");
    rows += e->ver_num[p];
  }
  return solve_common(e, list, rows, dist, pred, mode, stream);
}

int fap_solve_all(fap_engine *e, void *dist, int32_t *pred, void *stream) {
  return fap_solve(e, dist, pred, FAP_MODE_PLAIN, stream);
}

int fap_solve_batched(fap_engine *e, void *dist, int32_t *pred, void *stream) {
  return fap_solve(e, dist, pred, FAP_MODE_BATCHED, stream);
}

// Boundary marks and vertex order from graph_id (n entries, 1..K), and the
// device tables that depend on them; the engine's cached plans are dropped.
static int apply_partition(fap_engine *e, const int32_t *graph_id) {
  const int32_t n = e->n, K = e->K;
  for (int32_t i = 0; i < n; i++)
    if (graph_id[i] < 1 || graph_id[i] > K) return set_error(FAP_ERR_INVALID, "part id outside 1..K");
  std::vector<int32_t> gid(graph_id, graph_id + n), st2ed(n), ed2st(n);
  std::vector<int32_t> vn(K + 1), vo(K + 1), bn(K + 1), bo(K + 1);
  int rc = fapi::preprocess(K, n, gid.data(), e->ro.data(), e->col.data(), st2ed.data(), ed2st.data(),
                            vn.data(), vo.data(), bn.data(), bo.data(), nullptr);
  if (rc != FAP_OK) return rc;
  DeviceGuard g(e->device);
  // the plans and the device tables below may still be in use by work queued
  // on any stream (the engine's own, its side and copy streams, or a caller's
  // stream an earlier solve ran on): wait for the whole device first
  FAP_CUDA(cudaDeviceSynchronize());
  e->plans.clear();
  e->bg_ready = false;  // the boundary graph is rebuilt for the new parts on first use
  if (n > 0) {
    const size_t bytes = (size_t)n * sizeof(int32_t);
    FAP_CUDA(cudaMemcpy(e->d_gid, gid.data(), bytes, cudaMemcpyHostToDevice));
    FAP_CUDA(cudaMemcpy(e->d_st2ed, st2ed.data(), bytes, cudaMemcpyHostToDevice));
    FAP_CUDA(cudaMemcpy(e->d_ed2st, ed2st.data(), bytes, cudaMemcpyHostToDevice));
  }
  e->graph_id.swap(gid);
  e->st2ed.swap(st2ed);
  e->ed2st.swap(ed2st);
  e->ver_num.swap(vn);
  e->ver_offset.swap(vo);
  e->bdy_num.swap(bn);
  e->bdy_offset.swap(bo);
  return FAP_OK;
}

int fap_set_partition(fap_engine *e, const int32_t *graph_id) {
  if (!e || !graph_id) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  std::lock_guard<std::mutex> lk(e->mu);
  return apply_partition(e, graph_id);
}

int fap_precondition(fap_engine *e) {
  if (!e) return set_error(FAP_ERR_INVALID, "null argument");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  std::lock_guard<std::mutex> lk(e->mu);
  const std::vector<int32_t> gid = e->graph_id;
  return apply_partition(e, gid.data());
}

int fap_last_times(const fap_engine *e, double *times5) {
  if (!e || !times5) return set_error(FAP_ERR_INVALID, "null argument");
  for (int i = 0; i < 5; i++) times5[i] = e->times[i];
  return FAP_OK;
}

int fap_minplus_counters(fap_engine *e, uint64_t *out3, int32_t reset) {
  if (!e || !out3) return set_error(FAP_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  unsigned long long v[3] = {0, 0, 0};
  FAP_CUDA(fapk::strip_counters(v, reset != 0));
  for (int i = 0; i < 3; i++) out3[i] = v[i];
  return FAP_OK;
}

int fap_query(fap_engine *e, const void *dist, const int32_t *pred, int32_t nq, const int32_t *src,
              const int32_t *dst, void *out_dist, int32_t *out_len, int32_t *out_path, int32_t max_len,
              void *stream) {
  if (!e || nq < 0) return set_error(FAP_ERR_INVALID, "fap_query: bad arguments");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (nq == 0) return FAP_OK;
  if (!dist || !pred || !src || !dst || !out_dist || !out_len || (out_path && max_len < 1))
    return set_error(FAP_ERR_INVALID, "fap_query: null buffer");
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  fapi::clear_error();
  const void *bufs[] = {dist, pred, src, dst, out_dist, out_len};
  for (const void *b : bufs)
    if (!is_device_ptr(b)) return set_error(FAP_ERR_INVALID, "fap_query: buffers must be device memory");
  if (out_path && !is_device_ptr(out_path))
    return set_error(FAP_ERR_INVALID, "fap_query: out_path must be device memory");
  cudaStream_t st = pick_stream(e, stream);
  fapk::QueryArgs a{};
  a.n = e->n;
  a.dist = dist;
  a.pred = pred;
  a.ed2st = e->d_ed2st;
  a.nq = nq;
  a.src = src;
  a.dst = dst;
  a.out_dist = out_dist;
  a.out_len = out_len;
  a.out_path = out_path;
  a.max_len = max_len;
  a.status = e->d_status;
  FAP_CUDA(fapk::launch_query(e->f32(), a, st));
  FAP_CUDA(cudaStreamSynchronize(st));
  return check_status(e);
}

int fap_fw_counters(fap_engine *e, uint64_t *out2, int32_t reset) {
  if (!e || !out2) return set_error(FAP_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  unsigned long long strip = 0;
  FAP_CUDA(fapk::fw_strip_counter(&strip, reset != 0));
  out2[0] = strip;
  out2[1] = e->fw_host_work;
  if (reset) e->fw_host_work = 0;
  return FAP_OK;
}

int fap_last_launches(const fap_engine *e, int64_t *count) {
  if (!e || !count) return set_error(FAP_ERR_INVALID, "null argument");
  *count = e->last_launches;
  return FAP_OK;
}

int fap_minplus(fap_engine *e, int32_t dtype, int32_t M, int32_t N, int32_t K, const void *A,
                int64_t lda, const void *B, int64_t ldb, const int32_t *Bpath, int64_t ldbp,
                void *C, int64_t ldc, int32_t *Cpath, int64_t ldcp, void *stream) {
  if (!e || M < 0 || N < 0 || K < 0 || !C || (K > 0 && (!A || !B)))
    return set_error(FAP_ERR_INVALID, "fap_minplus: bad arguments");
  if (dtype != FAP_DTYPE_F32 && dtype != FAP_DTYPE_I32) return set_error(FAP_ERR_INVALID, "unknown dtype");
  if (Cpath == nullptr ? Bpath != nullptr : (Bpath == nullptr && K > 0))
    return set_error(FAP_ERR_INVALID, "Bpath and Cpath go together");
  if (lda < K || ldb < N || ldc < N || (Cpath && ldcp < N) || (Bpath && ldbp < N))
    return set_error(FAP_ERR_INVALID, "leading dimension too small");
  if (M == 0 || N == 0) return FAP_OK;
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  cudaStream_t st = pick_stream(e, stream);
  int tiles = 0;
  MpSegment s = mp_segment(A, lda, B, ldb, Bpath, ldbp, C, ldc, Cpath, ldcp, M, N, K, tiles);
  s.tile_begin = 0;
  s.strip_begin = 0;
  int rc;
  const bool i32 = dtype == FAP_DTYPE_I32;
  TableBuilder tb;
  size_t o_seg = tb.add(&s, 1);
  fapk::MatRef refs[2] = {{A, lda, M, K}, {B, ldb, K, N}};
  size_t o_ref = tb.add(refs, 2);
  if ((rc = e->small.ensure(tb.bytes.size())) != FAP_OK) return rc;
  FAP_CUDA(cudaMemcpyAsync(e->small.p, tb.bytes.data(), tb.bytes.size(), cudaMemcpyHostToDevice, st));
  unsigned char *base = static_cast<unsigned char *>(e->small.p);
  bool packed = false;
  if (i32 && K > 0) {
    // packed form only if max finite A + max finite B stays below the limit
    const fapk::MatRef *dr = reinterpret_cast<const fapk::MatRef *>(base + o_ref);
    FAP_CUDA(cudaMemsetAsync(e->d_status + 1, 0, 2 * sizeof(unsigned), st));
    FAP_CUDA(fapk::launch_max_finite(dr, 1, e->d_status + 1, st));
    FAP_CUDA(fapk::launch_max_finite(dr + 1, 1, e->d_status + 2, st));
    unsigned mx[2] = {0, 0};
    FAP_CUDA(cudaMemcpyAsync(mx, e->d_status + 1, sizeof(mx), cudaMemcpyDeviceToHost, st));
    FAP_CUDA(cudaStreamSynchronize(st));
    packed = (unsigned long long)mx[0] + mx[1] < fapk::pack_limit() &&
             (Cpath == nullptr || K <= fapk::max_packed_k());
  }
  const MpSegment *dseg = reinterpret_cast<const MpSegment *>(base + o_seg);
  // the strip form addresses C rows with 32-bit offsets within a 128-row strip
  if ((packed || (!i32 && K > 0)) && K <= fapk::minplus_strip_max_k() && ldc < (1 << 24) &&
      (!Cpath || ldcp < (1 << 24)))
    FAP_CUDA(fapk::launch_minplus_strips(Cpath != nullptr, dseg, 1, mp_strips_of(s), K, st, !i32,
                                         e->tile_cols, rows_aligned16(s)));
  else
    FAP_CUDA(fapk::launch_minplus_tiles(!i32, Cpath != nullptr, dseg, 1, tiles, packed, st));
  FAP_CUDA(cudaStreamSynchronize(st));
  return check_status(e);
}

int fap_fw_batched(fap_engine *e, int32_t dtype, int32_t count, const int32_t *sizes,
                   void *const *D, const int64_t *ld, int32_t *const *P, void *stream) {
  return fap_floyd_batched(e, dtype, count, sizes, D, ld, P, stream);
}

int fap_floyd_batched(fap_engine *e, int32_t dtype, int32_t count, const int32_t *sizes,
                      void *const *D, const int64_t *ld, int32_t *const *P, void *stream) {
  if (!e || count < 0 || (count > 0 && (!sizes || !D || !ld)))
    return set_error(FAP_ERR_INVALID, "fap_floyd_batched: bad arguments");
  if (dtype != FAP_DTYPE_F32 && dtype != FAP_DTYPE_I32) return set_error(FAP_ERR_INVALID, "unknown dtype");
  const bool pred = P != nullptr;
  const int Bk = fapk::fw_block();
  int maxnb = 0;
  for (int32_t b = 0; b < count; b++) {
    if (sizes[b] < 0 || ld[b] < sizes[b] || (sizes[b] > 0 && !D[b]) || (pred && sizes[b] > 0 && !P[b]))
      return set_error(FAP_ERR_INVALID, "fap_floyd_batched: bad matrix " + std::to_string(b));
    maxnb = std::max(maxnb, (sizes[b] + Bk - 1) / Bk);
  }
  if (count == 0 || maxnb == 0) return FAP_OK;
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  cudaStream_t st = pick_stream(e, stream);
  TableBuilder tb;
  std::vector<size_t> od(maxnb), op(maxnb), orr(maxnb), or2(maxnb), ops(maxnb), ols(maxnb);
  std::vector<int> nd(maxnb), np(maxnb), tp(maxnb), nr(maxnb), tr(maxnb), nr2(maxnb), sr2(maxnb), nps(maxnb),
      sps(maxnb), nls(maxnb), sls(maxnb);
  // tensor-map pairs of the matrices that meet the copy unit's alignment
  // rules (16-byte base and row stride); the others keep per-thread copies
  std::vector<int32_t> tmap1(count, 0);
  size_t o_tmaps = 0;
  bool has_tmaps = false;
  {
    std::vector<TmapBlob> maps;
    for (int32_t b = 0; b < count; b++) {
      TmapBlob two[2];
      if (sizes[b] > Bk && fapk::encode_fw_tmaps(two, D[b], pred ? P[b] : nullptr, ld[b], sizes[b], sizes[b])) {
        tmap1[b] = (int32_t)(maps.size() / 2) + 1;
        maps.push_back(two[0]);
        maps.push_back(two[1]);
      }
    }
    if (!maps.empty()) {
      o_tmaps = tb.add(maps.data(), maps.size());
      has_tmaps = true;
    }
  }
  for (int r = 0; r < maxnb; r++) {
    std::vector<FwDiagJob> dj;
    std::vector<MpSegment> ps, rs, r2s, pss, ls;
    int pt = 0, rt = 0, r2strips = 0, psstrips = 0, lstrips = 0;
    for (int32_t b = 0; b < count; b++) {
      int nb = (sizes[b] + Bk - 1) / Bk;
      if (r >= nb) continue;
      FwDiagJob j{};
      j.D = D[b];
      j.P = pred ? P[b] : nullptr;
      j.ld = ld[b];
      j.size = sizes[b];
      j.block = r;
      j.prev = r - 1;  // used by the packed form's pivot step (lookahead) only
      dj.push_back(j);
      if (nb > 1) {
        MpSegment a, c, rest;
        int t1, t2, t3;
        fw_segments(D[b], pred ? P[b] : nullptr, ld[b], sizes[b], r, a, c, rest, t1, t2, t3,
                    dtype == FAP_DTYPE_F32, tmap1[b]);
        if (dtype == FAP_DTYPE_F32 && r > 0)
          fw_look_strips(D[b], pred ? P[b] : nullptr, ld[b], sizes[b], r, nb, tmap1[b], ls, lstrips);
        a.tile_begin = pt;
        pt += t1;
        ps.push_back(a);
        c.tile_begin = pt;
        pt += t2;
        ps.push_back(c);
        rest.tile_begin = rt;
        rt += t3;
        rs.push_back(rest);
        fw_panel_strips(a, c, nb, pss, psstrips);
        MpSegment rest2 = rest;
        const int s2 = r + 1 < nb ? fw_rest_lookahead(rest2, nb, r) : fw_strips_of(rest, rest.tiles_x);
        if (s2 > 0) {
          rest2.strip_begin = r2strips;
          r2strips += s2;
          r2s.push_back(rest2);
        }
      }
    }
    nr2[r] = (int)r2s.size();
    sr2[r] = r2strips;
    or2[r] = tb.add(r2s.data(), r2s.size());
    nps[r] = (int)pss.size();
    sps[r] = psstrips;
    ops[r] = tb.add(pss.data(), pss.size());
    nls[r] = (int)ls.size();
    sls[r] = lstrips;
    ols[r] = tb.add(ls.data(), ls.size());
    nd[r] = (int)dj.size();
    od[r] = tb.add(dj.data(), dj.size());
    np[r] = (int)ps.size();
    tp[r] = pt;
    op[r] = tb.add(ps.data(), ps.size());
    nr[r] = (int)rs.size();
    tr[r] = rt;
    orr[r] = tb.add(rs.data(), rs.size());
  }
  const bool f32 = dtype == FAP_DTYPE_F32;
  std::vector<fapk::MatRef> refs;
  int32_t max_size = 0;
  for (int32_t b = 0; b < count; b++)
    if (sizes[b] > 0) {
      refs.push_back({D[b], ld[b], sizes[b], sizes[b]});
      max_size = std::max(max_size, sizes[b]);
    }
  size_t o_ref = tb.add(refs.data(), refs.size());
  int rc;
  if ((rc = e->small.ensure(std::max<size_t>(tb.bytes.size(), 64))) != FAP_OK) return rc;
  FAP_CUDA(cudaMemcpyAsync(e->small.p, tb.bytes.data(), tb.bytes.size(), cudaMemcpyHostToDevice, st));
  unsigned char *base = static_cast<unsigned char *>(e->small.p);
  const void *tmaps = has_tmaps ? static_cast<const void *>(base + o_tmaps) : nullptr;
  bool packed = false;
  if (!f32) {
    // a finite shortest distance is at most (size - 1) * the largest entry
    FAP_CUDA(cudaMemsetAsync(e->d_status + 1, 0, sizeof(unsigned), st));
    FAP_CUDA(fapk::launch_max_finite(reinterpret_cast<const fapk::MatRef *>(base + o_ref),
                                     (int)refs.size(), e->d_status + 1, st));
    unsigned mx = 0;
    FAP_CUDA(cudaMemcpyAsync(&mx, e->d_status + 1, sizeof(mx), cudaMemcpyDeviceToHost, st));
    FAP_CUDA(cudaStreamSynchronize(st));
    packed = (unsigned long long)mx * (unsigned long long)std::max(max_size - 1, 1) < fapk::pack_limit();
  }
  for (int r = 0; r < maxnb; r++) {
    const FwDiagJob *djobs = reinterpret_cast<const FwDiagJob *>(base + od[r]);
    if (packed) {  // lookahead, as in the solve's issue order
      if (r >= 2) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1 + r % 2], 0));
      FAP_CUDA(fapk::launch_fw_pivot(pred, djobs, nd[r], st));
      FAP_CUDA(cudaEventRecord(e->ev_fw[0], st));
      FAP_CUDA(cudaStreamWaitEvent(e->side, e->ev_fw[0], 0));
      FAP_CUDA(fapk::launch_fw_strips(pred, reinterpret_cast<const MpSegment *>(base + or2[r]), nr2[r],
                                      sr2[r], e->side, false, tmaps));
      FAP_CUDA(cudaEventRecord(e->ev_fw[1 + r % 2], e->side));
    } else if (f32) {  // FP32 lookahead, as in the solve's issue order
      if (r >= 2) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1 + r % 2], 0));
      if (nls[r] > 0)
        FAP_CUDA(fapk::launch_fw_strips(pred, reinterpret_cast<const MpSegment *>(base + ols[r]), nls[r],
                                        sls[r], st, true, tmaps));
      FAP_CUDA(fapk::launch_fw_diag(f32, pred, djobs, nd[r], st));
      if (nps[r] > 0)
        FAP_CUDA(fapk::launch_fw_strips(pred, reinterpret_cast<const MpSegment *>(base + ops[r]), nps[r],
                                        sps[r], st, true, tmaps));
      FAP_CUDA(cudaEventRecord(e->ev_fw[0], st));
      FAP_CUDA(cudaStreamWaitEvent(e->side, e->ev_fw[0], 0));
      if (nr2[r] > 0)
        FAP_CUDA(fapk::launch_fw_strips(pred, reinterpret_cast<const MpSegment *>(base + or2[r]), nr2[r],
                                        sr2[r], e->side, true, tmaps));
      FAP_CUDA(cudaEventRecord(e->ev_fw[1 + r % 2], e->side));
    } else {
      FAP_CUDA(fapk::launch_fw_diag(f32, pred, djobs, nd[r], st));
      {
        FAP_CUDA(fapk::launch_minplus_tiles(f32, pred, reinterpret_cast<const MpSegment *>(base + op[r]), np[r],
                                            tp[r], packed, st));
        FAP_CUDA(fapk::launch_minplus_tiles(f32, pred, reinterpret_cast<const MpSegment *>(base + orr[r]),
                                            nr[r], tr[r], packed, st));
      }
    }
  }
  if ((packed || f32) && maxnb > 0) FAP_CUDA(cudaStreamWaitEvent(st, e->ev_fw[1 + (maxnb - 1) % 2], 0));  // join
  FAP_CUDA(cudaStreamSynchronize(st));
  return check_status(e);
}

int fap_sssp(fap_engine *e, const int32_t *sources, int32_t num_sources, void *dist, int32_t *pred,
             int64_t ld, void *stream) {
  if (!e || num_sources < 0 || (num_sources > 0 && (!sources || !dist)))
    return set_error(FAP_ERR_INVALID, "fap_sssp: bad arguments");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (ld < e->n) return set_error(FAP_ERR_INVALID, "fap_sssp: ld < n");
  for (int32_t i = 0; i < num_sources; i++)
    if (sources[i] < 0 || sources[i] >= e->n) return set_error(FAP_ERR_INVALID, "fap_sssp: source out of range");
  if (num_sources == 0) return FAP_OK;
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard g(e->device);
  cudaStream_t st = pick_stream(e, stream);
  const bool acc64 = e->f32() && e->sssp_fp64;
  int lanes = e->sssp_lanes ? e->sssp_lanes
                            : fapk::sssp_lanes_for((num_sources + 7) / 8, (num_sources + 31) / 32, e->sm_count, acc64);
  if (acc64 && lanes == 8) lanes = 16;  // the FP64 search has no 8-source form
  const bool wide = acc64 && lanes == 32;
  std::vector<SsspBatch> batches;
  for (int b0 = 0; b0 < num_sources; b0 += lanes) {
    SsspBatch sb{};
    sb.count = std::min(lanes, num_sources - b0);
    for (int l = 0; l < sb.count; l++) {
      sb.src[l] = sources[b0 + l];
      sb.row_off[l] = (int64_t)(b0 + l) * ld;
    }
    batches.push_back(sb);
  }
  int rc;
  int slots = std::min((int)batches.size(), max_sssp_slots(e, wide));
  if ((rc = ensure_sssp_scratch(e, slots, wide)) != FAP_OK) return rc;
  if ((rc = e->small.ensure(batches.size() * sizeof(SsspBatch))) != FAP_OK) return rc;
  FAP_CUDA(cudaMemcpyAsync(e->small.p, batches.data(), batches.size() * sizeof(SsspBatch),
                           cudaMemcpyHostToDevice, st));
  fapk::SsspArgs sa{};
  sa.n = e->n;
  sa.ro = e->d_ro;
  sa.col = e->d_col;
  sa.w = e->d_w;
  sa.iro = e->d_iro;
  sa.icol = e->d_icol;
  sa.iw = e->d_iw;
  sa.batches = static_cast<const SsspBatch *>(e->small.p);
  sa.nbatches = (int)batches.size();
  sa.dist = dist;
  sa.pred = pred;
  sa.scratch = e->sssp_scratch.p;
  sa.slots = std::min(sa.nbatches, e->sssp_slots_alloc);
  sa.bits = e->sssp_bits.p;
  sa.status = e->d_status;
  sa.maxd = nullptr;
  sa.iter_cap = 8 * e->n + 64;
  sa.lanes = lanes;
  sa.acc64 = acc64;
  sa.delta = sssp_delta_of(e);
  FAP_CUDA(fapk::launch_sssp(e->f32(), sa, st));
  FAP_CUDA(cudaStreamSynchronize(st));
  return check_status(e);
}

int fap_backward(fap_engine *e, const int32_t *pred, int32_t num_pairs, const int32_t *s,
                 const int32_t *t, const float *g, float *dw, void *stream) {
  if (!e || num_pairs < 0 || (num_pairs > 0 && (!pred || !s || !t || !g || !dw)))
    return set_error(FAP_ERR_INVALID, "fap_backward: bad arguments");
  if (!e->has_graph) return set_error(FAP_ERR_STATE, "handle has no graph");
  if (!e->f32()) return set_error(FAP_ERR_INVALID, "fap_backward: FP32 engines only");
  if (num_pairs == 0) return FAP_OK;
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard dg(e->device);
  cudaStream_t st = pick_stream(e, stream);
  FAP_CUDA(fapk::launch_backward_graph(e->n, e->d_ro, e->d_col, static_cast<const float *>(e->d_w),
                                       e->d_ed2st, pred, num_pairs, s, t, g, dw, e->d_status, st));
  FAP_CUDA(cudaStreamSynchronize(st));
  return check_status(e);
}

int fap_backward_dense(fap_engine *e, int32_t count, const int32_t *sizes, int32_t *const *P,
                       float *const *dW, const int64_t *ld, int32_t num_pairs, const int32_t *b,
                       const int32_t *s, const int32_t *t, const float *g, void *stream) {
  if (!e || count < 0 || num_pairs < 0 || (count > 0 && (!sizes || !P || !dW || !ld)) ||
      (num_pairs > 0 && (!b || !s || !t || !g)))
    return set_error(FAP_ERR_INVALID, "fap_backward_dense: bad arguments");
  for (int32_t i = 0; i < count; i++)
    if (sizes[i] < 0 || ld[i] < sizes[i] || (sizes[i] > 0 && (!P[i] || !dW[i])))
      return set_error(FAP_ERR_INVALID, "fap_backward_dense: bad instance " + std::to_string(i));
  if (num_pairs == 0 || count == 0) return FAP_OK;
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard dg(e->device);
  cudaStream_t st = pick_stream(e, stream);
  const size_t rec = fapk::dense_inst_bytes();
  std::vector<unsigned char> tab(rec * count);
  for (int32_t i = 0; i < count; i++) fapk::fill_dense_inst(tab.data() + rec * i, P[i], dW[i], ld[i], sizes[i]);
  int rc;
  if ((rc = e->small.ensure(tab.size())) != FAP_OK) return rc;
  FAP_CUDA(cudaMemcpyAsync(e->small.p, tab.data(), tab.size(), cudaMemcpyHostToDevice, st));
  FAP_CUDA(fapk::launch_backward_dense(e->small.p, count, num_pairs, b, s, t, g, e->d_status, st));
  FAP_CUDA(cudaStreamSynchronize(st));
  return check_status(e);
}

int fap_addmin_peak(fap_engine *e, int32_t mode, double *ops_per_s) {
  if (!e || !ops_per_s || mode < 0 || mode > 12) return set_error(FAP_ERR_INVALID, "fap_addmin_peak: bad arguments");
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard dg(e->device);
  FAP_CUDA(fapk::measure_addmin_peak(mode, e->sm_count, ops_per_s));
  return FAP_OK;
}

int fap_set_option(fap_engine *e, int32_t option, double value) {
  if (!e) return set_error(FAP_ERR_INVALID, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  switch (option) {
    case FAP_OPT_SSSP_FP64:
      e->sssp_fp64 = value != 0.0 ? 1 : 0;
      return FAP_OK;
    case FAP_OPT_SSSP_DELTA:
      if (!(value >= 0.0) || std::isinf(value)) return set_error(FAP_ERR_INVALID, "SSSP delta must be >= 0");
      e->sssp_delta = (!e->f32() && value > 0.0) ? std::max(1.0, std::floor(value)) : value;
      return FAP_OK;
    case FAP_OPT_AUTOTUNE:
      e->autotune = value != 0.0 ? 1 : 0;
      return FAP_OK;
    case FAP_OPT_SSSP_LANES:
      if (value != 0.0 && value != 8.0 && value != 16.0 && value != 32.0)
        return set_error(FAP_ERR_INVALID, "SSSP lanes must be 0, 8, 16 or 32");
      e->sssp_lanes = (int)value;
      e->sssp_lanes_tuned = 0;
      return FAP_OK;
    case FAP_OPT_TILE_COLS:
      if (value != 0.0 && value != 64.0 && value != 128.0)
        return set_error(FAP_ERR_INVALID, "tile columns must be 0, 64 or 128");
      e->tile_cols = (int)value;
      return FAP_OK;
    case FAP_OPT_SSSP_METHOD:
      if (value != 0.0 && value != 1.0 && value != 2.0)
        return set_error(FAP_ERR_INVALID, "SSSP method must be 0, 1 or 2");
      e->sssp_method = (int)value;
      e->sssp_method_tuned = 0;
      return FAP_OK;
    case FAP_OPT_HOST_RESULTS:
      if (value != 0.0 && value != 1.0) return set_error(FAP_ERR_INVALID, "host results must be 0 or 1");
      e->host_results = (int)value;
      return FAP_OK;
    case FAP_OPT_INT32_FORM:
      if (value != 0.0 && value != 1.0) return set_error(FAP_ERR_INVALID, "int32 form must be 0 or 1");
      e->int32_form = (int)value;
      return FAP_OK;
    case FAP_OPT_HOST_GROUP_MB:
      if (!(value >= 1.0) || std::isinf(value)) return set_error(FAP_ERR_INVALID, "host group size must be >= 1 MB");
      e->host_group_mb = value;
      return FAP_OK;
    default:
      return set_error(FAP_ERR_INVALID, "unknown option");
  }
}

int fap_get_option(const fap_engine *e, int32_t option, double *value) {
  if (!e || !value) return set_error(FAP_ERR_INVALID, "null argument");
  switch (option) {
    case FAP_OPT_SSSP_FP64: *value = e->sssp_fp64; return FAP_OK;
    case FAP_OPT_SSSP_DELTA: *value = sssp_delta_of(e); return FAP_OK;
    case FAP_OPT_AUTOTUNE: *value = e->autotune; return FAP_OK;
    case FAP_OPT_SSSP_LANES: *value = e->sssp_lanes ? e->sssp_lanes : e->sssp_lanes_tuned; return FAP_OK;
    case FAP_OPT_TILE_COLS: *value = e->tile_cols; return FAP_OK;
    case FAP_OPT_SSSP_METHOD: *value = e->sssp_method ? e->sssp_method : e->sssp_method_tuned; return FAP_OK;
    case FAP_OPT_HOST_RESULTS: *value = e->host_results; return FAP_OK;
    case FAP_OPT_HOST_GROUP_MB: *value = e->host_group_mb; return FAP_OK;
    case FAP_OPT_INT32_FORM: *value = e->int32_form; return FAP_OK;
    default: return set_error(FAP_ERR_INVALID, "unknown option");
  }
}

int fap_sssp_stats(fap_engine *e, uint64_t *out5) {
  if (!e || !out5) return set_error(FAP_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(e->mu);
  DeviceGuard dg(e->device);
  unsigned long long h[8];
  FAP_CUDA(cudaMemcpy(h, e->d_stats, sizeof(h), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 5; i++) out5[i] = h[i];
  return FAP_OK;
}

}  // extern "C"
