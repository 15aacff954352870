// launch.h -- host-side launchers of the engine's CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace fapk {

// Kernel launches issued by this host thread (each launcher below adds the
// kernels it actually launches); plans record how many one solve issues.
int &launch_count();

// minplus.cu
// packed = true selects the packed int32 form (uint32 distances only); the
// caller must have checked that every finite result stays below
// pack_limit() and, with predecessors, that every segment has K <=
// max_packed_k().
// CTAs take tiles tile0 .. tile0 + tiles - 1 of the segments' numbering.
cudaError_t launch_minplus_tiles(bool f32, bool pred, const MpSegment *d_segs, int nseg,
                                 int tiles, bool packed, cudaStream_t st, int tile0 = 0);
// Strip form of the packed min-plus: segments that do not accumulate into C
// (init_from_c = 0), C's leading dimensions below 2^24, every
// K <= max_k <= minplus_strip_max_k(), CTAs numbered by
// MpSegment::strip_begin (ceil(M / 128) x ceil(tiles_x / minplus_strip_tiles())
// strips per segment).  Same preconditions as the packed tile form.
// f32: FP32 distances (any range) instead of the packed int32 form.
// tile_cols (packed form): 64 or 128-column tiles, 0 = the default of the
// K class (minplus_strip_class_cols); the FP32 form always takes 64.
// aligned: every segment's C (and Cp) rows start on 16-byte boundaries (the
// other form realigns its 16-byte stores row by row).
cudaError_t launch_minplus_strips(bool pred, const MpSegment *d_segs, int nseg, int strips,
                                  int max_k, cudaStream_t st, bool f32 = false, int tile_cols = 0,
                                  bool aligned = true);
int minplus_strip_class_cols(int c);
int minplus_strip_tiles();
// Strip form of the FW remaining-tile phase (packed int32, or FP32 with
// f32; init_from_c = 1, K <= 64): CTAs numbered by MpSegment::strip_begin,
// tiles_y x ceil(tiles_x / fw_strip_tiles()) strips per segment.  tmaps:
// device array of CUtensorMap pairs (distances, predecessors) indexed by
// MpSegment::tmap1 - 1 (64-byte aligned; null: no segment uses one).
cudaError_t launch_fw_strips(bool pred, const MpSegment *d_segs, int nseg, int strips,
                             cudaStream_t st, bool f32 = false, const void *tmaps = nullptr);
// Nonzero when a bulk tensor copy of the FW strips did not complete (the
// strip was abandoned: the results are not valid); optionally reset.
cudaError_t tma_status(unsigned *out, bool reset);
// Encodes the tensor-map pair of one 4-byte matrix (rows x cols, row
// stride ld elements) for the FW strips' 64 x 64 boxes into out[0] (d) and
// out[1] (p, or d again when p is null); false when the matrix does not meet
// the copy unit's alignment rules (16-byte base and row stride) or the
// driver has no encoder.
bool encode_fw_tmaps(void *out, const void *d, const void *p, int64_t ld, int rows, int cols);
int fw_strip_tiles();
int minplus_strip_max_k();   // largest K of the strip form
// Segments go to the strip form in classes of K (one launch per class, each
// with its own CTAs per SM): class c takes K <= minplus_strip_class_k(c)
// above the previous bound; -1 past the last class.
int minplus_strip_classes();
int minplus_strip_class_k(int c);
// Largest finite int32 entry of the matrices, atomicMax-ed into *out.
cudaError_t launch_max_finite(const MatRef *d_mats, int nmats, unsigned *out, cudaStream_t st);
unsigned pack_limit();
// Work counters of the strip min-plus on the current device: [tiles, tiles
// with no active step, active steps over all tiles]; optionally reset.
cudaError_t strip_counters(unsigned long long out[3], bool reset);
int max_packed_k();
// Add-mins executed by the FW remaining-tile strips on the current device
// since the last reset; optionally reset.
cudaError_t fw_strip_counter(unsigned long long *out, bool reset);
cudaError_t launch_fw_diag(bool f32, bool pred, const FwDiagJob *d_jobs, int njobs,
                           cudaStream_t st);
// Packed int32 form: closes each job's pivot block and updates its row and
// column panels (a cluster of CTAs per job); replaces launch_fw_diag and the
// panel launch.
cudaError_t launch_fw_pivot(bool pred, const FwDiagJob *d_jobs, int njobs, cudaStream_t st);
int minplus_tile_rows();  // CTA output tile edge (128)
int fw_block();           // FW pivot block edge (64)
cudaError_t init_minplus_kernels();

// sssp.cu
struct SsspArgs {
  int32_t n;
  const int32_t *ro, *col;    // out-edge CSR
  const void *w;              // out-edge weights (float or uint32)
  const int32_t *iro, *icol;  // in-edge CSR (for predecessors)
  const void *iw;
  const SsspBatch *batches;
  int32_t nbatches;
  void *dist;                 // output base (rows addressed by SsspBatch::row_off)
  int32_t *pred;              // may be null
  void *scratch;              // per-slot scratch, sssp_slot_bytes(n, acc64 && lanes == 32) each
  int32_t slots;              // number of CTAs (= scratch slots)
  void *bits;                 // slots * sssp_bits_bytes(n): frontier bitmaps that do
                              // not fit in shared memory (null when that is 0)
  unsigned *status;           // device status word (error flags are or-ed in)
  unsigned *maxd;             // largest finite int32 distance written (atomicMax), may be null
  int32_t iter_cap;           // steps (near-frontier sweeps + far splits) per batch
  int32_t lanes;              // sources per batch: 8, 16 or 32 (batches hold <= lanes;
                              // 16 or 32 with acc64)
  int32_t acc64;              // FP32 weights searched in FP64 (8-byte entries)
  double delta;               // near-far threshold step (> 0; huge = plain Bellman-Ford)
  unsigned long long *stats;  // may be null: [near steps, far splits, frontier
                              // vertices relaxed, far entries scanned, batches]
  int32_t defer_output;       // set by launch_sssp: output pass in its own launch
  // launch_sssp_output on tables of exact 64-bit fixed point (FP32 graphs):
  int32_t fix;                        // 1: tables hold fixed-point values, not FP64
  const unsigned long long *iwfix;    // in-edge weights in the same units
  unsigned long long fix_inf;         // values at or above are unreached
  double fix_scale;                   // 2^-shift: fixed point -> distance
};
// delta value that puts every vertex in the near frontier (plain frontier BF)
constexpr double kSsspNoDelta = 2147483647.0;
cudaError_t init_sssp_kernels();
size_t sssp_slot_bytes(int32_t n, bool wide = false);  // wide: FP64 search with 32 lanes
size_t sssp_bits_bytes(int32_t n);  // per slot; 0 when the bitmaps fit in shared memory
// Batch width (8, 16 or 32 sources) given the batches the work needs at 8 and 32.
int sssp_lanes_for(int64_t batches8, int64_t batches32, int sm_count, bool acc64);
int sssp_threads();
cudaError_t launch_sssp(bool f32, const SsspArgs &a, cudaStream_t st);

// Output pass of the whole-graph search alone, over per-batch vertex-major
// tables that something else filled (batch b's table in scratch slot b,
// a.slots >= a.nbatches): predecessors, rounding, row stores.  acc64: FP32
// graphs with FP64 tables (8-byte entries, 16 or 32 lanes).
cudaError_t launch_sssp_output(bool f32, const SsspArgs &a, cudaStream_t st);

// bgraph.cu -- boundary SSSP through the boundary graph (exact arithmetic:
// uint32 for int32 graphs, 64-bit fixed point for FP32 graphs ("wide")).
struct BgPart {
  int32_t start;  // first sorted position of the part
  int32_t sub, bdy;
  int32_t boff;   // boundary index of its first boundary vertex
  int64_t loff;   // element offset of its local rows (bdy x sub) in the L arena
};
struct BgJob {    // step 1: (part, first local source, count); step 2: (batch, first lane, count)
  int32_t unit, first, count;
};
struct BgArgs {
  int32_t nparts;
  const BgPart *parts;
  int32_t B;                   // boundary vertices = nodes of the boundary graph
  const int32_t *bpart;        // [B] part (index into parts) of each boundary node
  const int32_t *lro;          // [n + 1] by sorted position: local out-edges of the vertex
  const int32_t *lcol;         // local index (within its part) of the edge's target
  const void *lw;              // edge weights (uint32 or 64-bit fixed point)
  const int32_t *cro;          // [B + 1] cut out-edges of each boundary node
  const int32_t *ccol;         // boundary index of the target
  const void *cw;              // weights
  const BgJob *ljobs;          // step-1 jobs
  const BgJob *bjobs;          // step-2 jobs
  const int32_t *bsrc;         // [batches][32] boundary index of each SSSP source (-1: none)
  void *L;                     // local rows of every part
  void *DS;                    // [B][B] boundary-graph distances, row = source boundary index
  unsigned *status;
  unsigned long long *stats;   // may be null: [rounds, -, nodes visited, -, -]
  // threshold steps of the distance-ordered frontier (0: plain Bellman-Ford),
  // in the weights' units, for steps 1 and 2
  unsigned long long delta_local, delta_boundary;
};
struct BgRowArgs {
  const SsspBatch *batches;
  int32_t nbatches;
  const int32_t *st2ed;
  void *scratch;               // batch b's table at scratch + b * slot_bytes
  size_t slot_bytes;
  unsigned long long fix_inf;  // wide tables: entries at or above are unreached (written as fix_inf)
};
constexpr size_t kBgSmemMax = 226 * 1024;  // dynamic; the 227 KB per-block limit also holds the static part
size_t bg_smem_bytes(bool wide, int nodes);  // shared memory of steps 1 and 2 over `nodes` nodes
int bg_lanes();                              // sources per CTA in steps 1 and 2
cudaError_t init_bg_kernels();
cudaError_t launch_bg_local(bool wide, const BgArgs &a, int njobs, int max_sub, cudaStream_t st);
cudaError_t launch_bg_boundary(bool wide, const BgArgs &a, int njobs, cudaStream_t st);
cudaError_t launch_bg_rows(bool wide, int lanes, const BgArgs &a, const BgRowArgs &r, cudaStream_t st);

// query.cu -- point-to-point queries on solve() rows in device memory
struct QueryArgs {
  int32_t n;
  const void *dist;        // n x n solve() rows (row = sorted position)
  const int32_t *pred;
  const int32_t *ed2st;    // vertex -> row
  int32_t nq;
  const int32_t *src, *dst;
  void *out_dist;          // nq entries of the distance type
  int32_t *out_len;        // vertices on each path (0: unreached)
  int32_t *out_path;       // nq x max_len, may be null
  int32_t max_len;
  unsigned *status;
};
cudaError_t launch_query(bool f32, const QueryArgs &a, cudaStream_t st);

// transform.cu
struct PartDesc {
  int32_t sub, bdy, start;  // part size, boundary count, first sorted position
  int32_t ld;               // leading dimension of the part's FW matrix
  int64_t mat_off;          // element offset of the FW matrix in the arena
  int64_t row_off;          // element offset of the part's first boundary row (SSSP output, build input)
  int64_t dec_off;          // element offset of the part's first row where the decode writes
};
struct BuildArgs {
  int32_t n;
  const int32_t *ro, *col;
  const void *w;
  const int32_t *graph_id, *st2ed, *ed2st;
  const PartDesc *parts;
  const int64_t *row_begin;  // prefix sums of padded rows per part (nparts+1)
  const int64_t *dec_begin;  // prefix sums of boundary rows per part (nparts+1)
  int32_t nparts;
  int64_t total_rows;
  int64_t dec_rows;
  void *mat;                 // FW matrices arena (dist)
  int32_t *matp;             // FW matrices arena (pred), may be null
  const void *rows;          // result rows (dist), source of boundary rows
  const int32_t *rowsp;      // result rows (pred)
  int64_t ldr;               // leading dimension of the result rows (n)
};
cudaError_t launch_build(bool f32, bool pred, const BuildArgs &a, cudaStream_t st);
cudaError_t launch_decode(bool f32, bool pred, const BuildArgs &a, void *rows, int32_t *rowsp,
                          cudaStream_t st);

// adjoint.cu
cudaError_t launch_backward_graph(int32_t n, const int32_t *ro, const int32_t *col, const float *w,
                                  const int32_t *ed2st, const int32_t *pred, int32_t npairs,
                                  const int32_t *s, const int32_t *t, const float *g, float *dw,
                                  unsigned *status, cudaStream_t st);
cudaError_t launch_backward_dense(const void *inst, int32_t ninst, int32_t npairs,
                                  const int32_t *b, const int32_t *s, const int32_t *t,
                                  const float *g, unsigned *status, cudaStream_t st);
size_t dense_inst_bytes();
void fill_dense_inst(void *dst, const int32_t *P, float *dW, int64_t ld, int32_t size);

// probe.cu
cudaError_t measure_addmin_peak(int mode, int sm_count, double *ops_per_s);

}  // namespace fapk
