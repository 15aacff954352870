/*
 * fastapsp.h -- C ABI of the GB300 Fast-APSP engine.
 *
 * The engine computes all-pairs shortest paths by the divide-and-conquer
 * method of TomerHaham/FastAPSP: the vertex set is split into K parts on the
 * host; per part, an SSSP runs from every boundary vertex over the whole
 * graph, a Floyd-Warshall closes the part's dense sub x sub matrix, and a
 * (min,+) product extends the inner rows to every vertex.  The hot path runs as
 * hand-written sm_103a CUDA kernels on one GPU.
 *
 * Conventions
 *  - Every function returns an int status: FAP_OK (0) or a negative FAP_ERR_*
 *    code.  Nothing calls exit(); fap_last_error() gives a message.
 *  - Vertex ids are 0-based; part ids are 1-based (1..K), as in the reference
 *    (fap/utils/readIdFile.h:279-283).
 *  - Distances are FP32 (unreached = 1e8, FAP_MAXVALUE_F32, as
 *    fap/utils/parameter.h:26) or int32 (unreached = 2^30, FAP_INF_I32).
 *    Predecessors are int32 original vertex ids, -1 = unreached, and
 *    pred[s][s] = s.
 *  - Result rows follow the reference layout (fap/fap.cpp:507-518,
 *    fap/utils/util_Myalgorithm.h:236-247): the rows of part i are the part's
 *    vertices in mapping (st2ed) order -- boundary vertices first -- and the
 *    columns are original vertex ids.  solve() stacks the parts 1..K.
 *  - Result buffers may be host memory (pageable or pinned) or device memory
 *    of the engine's GPU; the engine detects which.  Streams are passed as
 *    `void *` (a cudaStream_t) so that this header needs no CUDA headers;
 *    NULL means the engine's own stream.  Work issued on a caller's stream
 *    is ordered on that stream: the Floyd-Warshall phase of the packed int32
 *    form forks part of its launches to an internal stream of the engine
 *    and joins it back on the caller's stream before the next phase.
 */
#ifndef FASTAPSP_H_
#define FASTAPSP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define FAP_OK 0
#define FAP_ERR_INVALID (-1)       /* bad argument */
#define FAP_ERR_CUDA (-2)          /* a CUDA runtime call failed */
#define FAP_ERR_NOMEM (-3)         /* device or host allocation failed */
#define FAP_ERR_STATE (-4)         /* call not valid in the handle's state */
#define FAP_ERR_NOT_CONVERGED (-5) /* SSSP hit its iteration cap */
#define FAP_ERR_IO (-6)            /* file could not be read */
#define FAP_ERR_NO_DEVICE (-7)     /* no CUDA device / wrong architecture */
#define FAP_ERR_RANGE (-8)         /* value outside the supported range */

#define FAP_DTYPE_F32 0
#define FAP_DTYPE_I32 1

#define FAP_MAXVALUE_F32 1e8f
#define FAP_INF_I32 0x40000000

/* Solve modes. */
#define FAP_MODE_PLAIN 0   /* one launch sequence per part, parts in order */
#define FAP_MODE_BATCHED 1 /* all parts per phase launch, in a CUDA graph */

typedef struct fap_engine fap_engine; /* opaque */

/* ---- library ------------------------------------------------------------ */
const char *fap_version(void);
const char *fap_status_string(int status);
/* Message of the last failing call on this thread ("" if none). */
const char *fap_last_error(void);
/* Number of usable CUDA devices (0 without a GPU; never fails). */
int fap_device_count(int32_t *count);

/* ---- host preprocessing (CPU only, no GPU needed) ------------------------ */

/* Replaces readVerEdges (fap/utils/readMatFile.h:36-64): vertex count and
 * CSR entry count (doubled for undirected input) from a MatrixMarket
 * header.  `path` is the full path of the .mtx file. */
int fap_mtx_counts(const char *path, int32_t directed, int32_t weighted,
                   int32_t *n, int64_t *m);

/* Replaces readMatFile (fap/utils/readMatFile.h:66-173): CSR with 1-based
 * input ids, undirected lines doubled, |w| for weighted input, w = 1 for
 * unweighted input, duplicates and self loops kept, each row in reverse input
 * order.  Arrays sized from fap_mtx_counts: adj_size[n], row_offset[n+1],
 * col_val[m], weight[m]. */
int fap_mtx_read(const char *path, int32_t directed, int32_t weighted,
                 int32_t n, int64_t m, int32_t *adj_size, int32_t *row_offset,
                 int32_t *col_val, float *weight);

/* Replaces readIdFile_METIS / Graph_decomposition
 * (fap/utils/readIdFile.h:79-304): K-way partition of the symmetrized graph
 * by the engine's multilevel partitioner (heavy-edge coarsening, greedy
 * growing bisection, boundary refinement; 3% imbalance).  Writes 1-based part
 * ids into graph_id[n]; edge_cut (nullable) receives the number of cut
 * undirected edges. */
int fap_partition(int32_t n, const int32_t *row_offset, const int32_t *col_val,
                  int32_t K, uint64_t seed, int32_t *graph_id,
                  int64_t *edge_cut);

/* Replaces findBoundry + sort_and_encode (fap/utils/util_preprocess.h:32-106):
 * boundary marks (both endpoints of every cross-part CSR entry), the vertex
 * order (part ascending, boundary first; st2ed[pos] = original id, ed2st its
 * inverse) and the per-part counts/offsets ver_num, ver_offset, bdy_num,
 * bdy_offset (K+1 entries each, index 0 unused).  The order inside a
 * (part, boundary) group is that of the reference's std::sort call. */
int fap_preprocess(int32_t K, int32_t n, const int32_t *graph_id,
                   const int32_t *row_offset, const int32_t *col_val,
                   int32_t *st2ed, int32_t *ed2st, int32_t *ver_num,
                   int32_t *ver_offset, int32_t *bdy_num, int32_t *bdy_offset);

/* ---- engine: one graph on one GPU --------------------------------------- */

/* Replaces fapGraph(num_vertexs, num_edges, row_offset, col_val, weight, K)
 * (fap/fap.h:102-104; empty in the reference, fap/fap.cpp:94-98) followed by
 * preCondition() (fap/fap.cpp:100-114).  Copies the CSR (row_offset[n+1],
 * col_val[m], weight[m]) to device `device`.  graph_id (n, 1-based) may be
 * NULL, in which case fap_partition(seed 1) supplies it.  dtype selects the
 * distance arithmetic: FAP_DTYPE_F32 (weights used as given) or
 * FAP_DTYPE_I32 (non-negative integer weights with (n-1) * max weight below
 * 2^30, so that no finite distance reaches the int32 "unreached" value). */
int fap_create(int32_t n, int64_t m, const int32_t *row_offset,
               const int32_t *col_val, const float *weight, int32_t K,
               const int32_t *graph_id, int32_t dtype, int32_t device,
               fap_engine **out);

/* A handle without a graph, for the standalone kernels below. */
int fap_create_context(int32_t device, fap_engine **out);

int fap_destroy(fap_engine *e);

/* Metadata getters (fap/fap.cpp:546-566, 640-670).  Arrays are copied. */
int fap_num_vertices(const fap_engine *e, int32_t *n, int32_t *K);
int fap_mapping(const fap_engine *e, int32_t *st2ed);     /* n entries */
int fap_graph_id(const fap_engine *e, int32_t *graph_id); /* n entries */
/* sub = C_BlockVer_num[part], bdy = C_BlockBdy_num[part],
 * offset = C_BlockVer_offset[part]. */
int fap_part_info(const fap_engine *e, int32_t part, int32_t *sub,
                  int32_t *bdy, int32_t *offset);

/* Replaces solveSubGraph(id) (fap/fap.cpp:520-545) and the per-part
 * pipeline fapGraph::run (fap/fap.cpp:195-503): writes the part's sub x n
 * rows (dist of the engine dtype, pred int32; pred may be NULL). */
int fap_solve_part(fap_engine *e, int32_t part, void *dist, int32_t *pred,
                   void *stream);

/* Replaces solve() (fap/fap.cpp:507-518): all parts, n x n rows stacked by
 * part.  mode = FAP_MODE_PLAIN (per-part launch sequences, like the
 * reference's host loop) or FAP_MODE_BATCHED (every phase runs over all parts
 * in one launch; the launch sequence is replayed from a CUDA graph). */
int fap_solve(fap_engine *e, void *dist, int32_t *pred, int32_t mode,
              void *stream);

/* Several parts in one call (no single reference counterpart: the
 * reference's MPI task layer runs solveSubGraph over each process's parts,
 * fap/fap_more_task_mpi.cpp:34-91): the rows of parts[0..nparts) go to
 * dist/pred one part after another in the order listed, each part's rows in
 * mapping order (sub_i x n each); mode as fap_solve (FAP_MODE_BATCHED: one
 * launch per phase over all listed parts).  This is what a process of a
 * part-sharded multi-GPU run calls with its share of the parts.  Parts must
 * be distinct, 1..K. */
int fap_solve_parts(fap_engine *e, const int32_t *parts, int32_t nparts,
                    void *dist, int32_t *pred, int32_t mode, void *stream);

/* fap_solve in each mode by name: solve() part by part
 * (fap/fap.cpp:507-518), and the batched form. */
int fap_solve_all(fap_engine *e, void *dist, int32_t *pred, void *stream);
int fap_solve_batched(fap_engine *e, void *dist, int32_t *pred, void *stream);

/* Replaces the partition the fapGraph constructor reads
 * (fap/utils/readIdFile.h:79-304 fills graph_id) for an existing engine:
 * graph_id (n entries, 1..K, host memory) becomes the engine's partition and
 * the boundary marks and vertex order are recomputed as in fap_precondition;
 * cached plans are dropped, later solves use the new parts.  Do not call it
 * while another call on this engine is in flight. */
int fap_set_partition(fap_engine *e, const int32_t *graph_id);

/* Replaces fapGraph::preCondition() (fap/fap.cpp:100-114: findBoundry and
 * sort_and_encode, fap/utils/util_preprocess.h:32-106) on an engine:
 * recomputes the boundary marks and the vertex order (fap_mapping) from the
 * engine's partition.  fap_create already does it; the call is idempotent. */
int fap_precondition(fap_engine *e);

/* Engine options (no reference counterpart).
 *   FAP_OPT_SSSP_FP64  (FP32 engines) 1 = run the boundary SSSP in exact or
 *                      FP64 arithmetic and round once to FP32, which keeps
 *                      results within an ulp or two of FP64 shortest
 *                      distances on long paths; 0 (default) = FP32
 *                      arithmetic, bit-identical to the reference's FP32
 *                      Dijkstra.
 *   FAP_OPT_SSSP_DELTA near-far threshold step of the SSSP in distance units
 *                      (0 = automatic).  Changes speed only, never results.
 *   FAP_OPT_AUTOTUNE   1 (default) = while the step is automatic, the first
 *                      run of a solve times the SSSP phase with a few steps
 *                      (multiples of the mean edge weight, and plain
 *                      Bellman-Ford) and keeps the fastest; fap_get_option
 *                      then reports the chosen step.  0 = 8 x the mean weight.
 *   FAP_OPT_SSSP_LANES sources per SSSP batch (one CTA each; 8 = four lane
 *                      groups a warp, 16 = two, 32 = one): 8, 16 or 32, or 0
 *                      (default) = automatic: chosen from the batch count,
 *                      and while the step is tuned (above), the first run
 *                      also times a second width at the chosen step and
 *                      keeps the faster, which fap_get_option then reports
 *                      (not with FAP_OPT_SSSP_FP64, which takes 16 unless 32
 *                      is set).  Changes speed only, never results.
 *   FAP_OPT_TILE_COLS  column width of the packed int32 min-plus tiles (128
 *                      rows): 64 or 128, or 0 (default) = chosen per K class
 *                      of each plan: while FAP_OPT_AUTOTUNE is on, the first
 *                      run times both widths and keeps the faster (not for
 *                      results in mapped host memory); otherwise 64 for
 *                      K <= 48 and 128 above.  Changes speed only.
 *   FAP_OPT_SSSP_METHOD how the boundary SSSP rows of a solve are made.
 *                      The boundary-graph method (local rows of every part
 *                      from its boundary vertices, shortest paths between
 *                      all boundary vertices over the cut edges and those
 *                      rows, then a min-plus per part) applies where its
 *                      arithmetic is exact -- int32 engines, and FP32
 *                      engines with FAP_OPT_SSSP_FP64 whose weights are
 *                      multiples of one power of two 2^-s with
 *                      (n-1) * max weight < 2^(52-s) (64-bit fixed point) --
 *                      and its tables fit in shared memory (up to about
 *                      3,200 boundary vertices for FP32, 5,800 for int32);
 *                      elsewhere the whole-graph search runs.  0 (default)
 *                      = automatic: while FAP_OPT_AUTOTUNE is on, the first
 *                      run of a plan where the boundary graph applies times
 *                      both methods and keeps the faster (fap_get_option
 *                      then reports 1 or 2); 1 = always the whole-graph
 *                      search; 2 = the boundary graph wherever it applies.
 *                      Both give the same distances (int32: identical;
 *                      FP32: the exactly rounded distance, which equals the
 *                      FP64 search's whenever its sums are exact) and the
 *                      same predecessor rule.
 *   FAP_OPT_HOST_RESULTS results in page-locked host memory: 0 (default) =
 *                      solved into a device copy that the copy engines then
 *                      move to the host rows, when the device has room for
 *                      it; 1 = the kernels store the inner rows straight
 *                      into the host rows (no device copy of the n x n
 *                      result; also the choice of 0 without room).  Same
 *                      rows either way.
 *   FAP_OPT_INT32_FORM (int32 engines) 0 (default) = the FW and min-plus run
 *                      on packed keys (distance << 7 | step, one DPX add-min)
 *                      when the first run of a plan proves every finite
 *                      result stays below 2^24 - 1, else on separate values
 *                      and steps (the wide form); 1 = always the wide form.
 *                      Same rows either way.
 *   FAP_OPT_HOST_GROUP_MB results in page-locked host memory, batched solves:
 *                      the parts are solved in groups of about this many MB
 *                      of result rows (default 8192; at most 8 groups), each
 *                      group's rows copied out while the next group computes.
 *                      FP32 engines with three or more groups hold the
 *                      device copy in two group-sized slots that the groups
 *                      take in turn.  Same rows for any value.
 * Setting an option takes effect from the next solve. */
#define FAP_OPT_SSSP_FP64 1
#define FAP_OPT_SSSP_DELTA 2
#define FAP_OPT_AUTOTUNE 3
#define FAP_OPT_SSSP_LANES 4
#define FAP_OPT_TILE_COLS 5
#define FAP_OPT_SSSP_METHOD 6
#define FAP_OPT_HOST_RESULTS 7
#define FAP_OPT_INT32_FORM 8
#define FAP_OPT_HOST_GROUP_MB 9
int fap_set_option(fap_engine *e, int32_t option, double value);
int fap_get_option(const fap_engine *e, int32_t option, double *value);

/* Device time of the last solve's phases in milliseconds:
 * [sssp, floyd, min_plus, data, total] (the getTime* counters of
 * fap/fap.cpp:622-639, measured with CUDA events). */
int fap_last_times(const fap_engine *e, double *times5);
/* Number of kernels the last solve launched (no reference counterpart; the
 * bench reports it as the GPU launch count of a step). */
int fap_last_launches(const fap_engine *e, int64_t *count);
/* Work counters of the min-plus strip kernel on the engine's GPU since the
 * last reset (no reference counterpart; diagnostics of the sparsity skip):
 * [tiles, tiles with no active k-step, add-mins executed: active k-steps x
 * the tile's outputs (128 x 64 or 128 x 128), summed over tiles].  reset != 0
 * clears them after reading. */
int fap_minplus_counters(fap_engine *e, uint64_t *out3, int32_t reset);
/* Floyd-Warshall work of the solves since the last reset (no reference
 * counterpart; the executed-work view of the FW roofline): [add-mins the
 * remaining-tile strips executed on the engine's GPU (steps they ran x tile
 * outputs; they skip steps whose pivot row or column is unreached over the
 * tile), add-mins of the other FW launches (the pivot steps' 64 x 64 x 64
 * block products in the packed int32 form, every block in the other forms,
 * which skip nothing)].  reset != 0 clears them after reading. */
int fap_fw_counters(fap_engine *e, uint64_t *out2, int32_t reset);

/* ---- standalone kernels on caller device memory ------------------------- */

/* Replaces min_plus_path_advanced_gpu (fap/kernel/minplus.h:81-90,
 * minplus_NVIDIA_path_gpu, fap/kernel/cuda/minplus.cu:268-359):
 *   C[i][j] = min_k A[i][k] + B[k][j],  Cpath[i][j] = Bpath[k*][j]
 * for i < M, j < N, k < K, with k* the first k that reaches the minimum and
 * C = unreached / Cpath = -1 where no k gives a finite sum.  All pointers are
 * device memory, row-major with the given leading dimensions (elements).
 * Bpath and Cpath may both be NULL (distances only). */
int fap_minplus(fap_engine *e, int32_t dtype, int32_t M, int32_t N, int32_t K,
                const void *A, int64_t lda, const void *B, int64_t ldb,
                const int32_t *Bpath, int64_t ldbp, void *C, int64_t ldc,
                int32_t *Cpath, int64_t ldcp, void *stream);

/* Replaces floyd_path_gpu (fap/kernel/floyd.h:150-158,
 * floyd_GPU_Nvidia_path_gpu, fap/kernel/cuda/floyd.cu:286-342): in-place
 * Floyd-Warshall of `count` independent square matrices in one batched launch
 * sequence.  D[b] is sizes[b] x sizes[b] with leading dimension ld[b]; P[b]
 * (same shape and leading dimension, may be NULL for all b) is updated as
 * P[i][j] = P[k][j] on every strict improvement.  The pointer arrays live in
 * host memory; the matrices in device memory. */
int fap_floyd_batched(fap_engine *e, int32_t dtype, int32_t count,
                      const int32_t *sizes, void *const *D, const int64_t *ld,
                      int32_t *const *P, void *stream);
/* The same call under the name fap_fw_batched. */
int fap_fw_batched(fap_engine *e, int32_t dtype, int32_t count,
                   const int32_t *sizes, void *const *D, const int64_t *ld,
                   int32_t *const *P, void *stream);

/* Replaces handle_boundry_path_data_on_gpu (fap/kernel/batch_sssp.h:254-278,
 * multi_source_Nvidia_sssp_data_on_gpu, fap/kernel/cuda/batch_sssp.cu:
 * 361-414): SSSP from `num_sources` vertices (host array) of the engine's
 * graph; row r of dist/pred (device memory, leading dimension ld) receives
 * the distances/predecessors from sources[r].  Predecessors follow the
 * reference's Dijkstra (batch_sssp.h:79-114): among the in-neighbours u of v
 * whose relaxation reaches dist[v], the one first in (dist[u], u) order. */
int fap_sssp(fap_engine *e, const int32_t *sources, int32_t num_sources,
             void *dist, int32_t *pred, int64_t ld, void *stream);

/* Adjoint of the APSP distances with respect to the edge weights (no
 * reference counterpart).  For each (s[i], t[i], g[i]) triple, g[i] is added
 * to dw[e] for every CSR entry e on the predecessor path from s[i] to t[i]
 * (the lightest entry u->v of each step).  pred holds full n x n rows in
 * solve() layout (row of vertex s = its mapping position); pred, s, t, g and
 * dw (m entries, accumulated into) are device memory.  Unreached pairs add
 * nothing. */
int fap_backward(fap_engine *e, const int32_t *pred, int32_t num_pairs, const int32_t *s,
                 const int32_t *t, const float *g, float *dw, void *stream);

/* Adjoint for batches of dense instances (no reference counterpart): for each
 * (b[i], s[i], t[i], g[i]), g[i] is added to dW[b][u][v] for every step u->v
 * of the predecessor path from s[i] to t[i] in instance b.  P[b] and dW[b]
 * are device matrices of sizes[b] x sizes[b] with leading dimension ld[b]
 * (the P matrices of fap_floyd_batched); the pointer arrays live in host
 * memory; b, s, t, g are device arrays. */
int fap_backward_dense(fap_engine *e, int32_t count, const int32_t *sizes,
                       int32_t *const *P, float *const *dW, const int64_t *ld,
                       int32_t num_pairs, const int32_t *b, const int32_t *s,
                       const int32_t *t, const float *g, void *stream);

/* Allocation-free batched SSSP (no counterpart in the reference).  For
 * callers that cannot call cudaMalloc -- code running under an allocator it
 * does not own (a framework's memory pool or arena), request paths of
 * plugins whose host forbids allocation, real-time paths that cannot take an
 * allocation's latency or implicit synchronization.  Same kernel and same
 * results as fap_sssp, but without an engine handle: the caller passes the
 * graph in device memory it owns -- the out-edge CSR (row_offset[n+1],
 * col_val[m], weight[m]) and, when pred is not NULL, the in-edge CSR -- with
 * 4-byte weights (float for FAP_DTYPE_F32, int32 for FAP_DTYPE_I32), the
 * sources in host memory, and device rows dist/pred of num_sources x ld.
 * All scratch comes from one static device array of FAP_NOALLOC_SCRATCH_BYTES
 * (64 MiB) that every GPU loading this library holds until exit; graphs whose
 * scratch does not fit (about n > 460,000 vertices) are rejected with
 * FAP_ERR_RANGE.  No allocation: neither cudaMalloc/cudaFree nor an
 * allocating library call.  The first call on a device looks up the array's
 * device address and raises the SSSP kernels' shared-memory limits there (so
 * make that first call before any stream capture); no engine is needed.  Calls
 * share the array: each call clears what must start at zero, and calls that
 * overlap on the GPU race, so serialize them.  The call synchronizes
 * `stream` before returning its status. */
#define FAP_NOALLOC_SCRATCH_BYTES (64u << 20)
int fap_sssp_noalloc(int32_t dtype, int32_t n, int64_t m,
                     const int32_t *row_offset, const int32_t *col_val,
                     const void *weight, const int32_t *in_row_offset,
                     const int32_t *in_col_val, const void *in_weight,
                     const int32_t *sources, int32_t num_sources, void *dist,
                     int32_t *pred, int64_t ld, void *stream);

/* Point-to-point queries on the rows of a full fap_solve kept in device
 * memory (no reference counterpart: the reference declares getDistanceP2P /
 * getPathP2P, fap/fap.h:144-145, without bodies, fap/fap.cpp:674-680, and
 * keeps its results in host vectors).  dist / pred: the n x n solve() rows
 * on the engine's GPU (row r = vertex mapping[r], columns = vertex ids);
 * src[nq] / dst[nq]: vertex ids; all buffers device memory.  For query q:
 * out_dist[q] = the distance (int32 or float like dist; the unreached
 * sentinel when there is no path), out_len[q] = vertices on the path
 * src..dst (1 when src == dst, 0 when unreached), and, when out_path is not
 * NULL, that path in out_path[q * max_len ...] when it has at most max_len
 * vertices (a longer path reports its length and leaves its slots as they
 * were).  Ids outside 0..n-1, or predecessors that do not lead back to src
 * within n steps, give FAP_ERR_INVALID.  Synchronizes `stream`. */
int fap_query(fap_engine *e, const void *dist, const int32_t *pred, int32_t nq,
              const int32_t *src, const int32_t *dst, void *out_dist,
              int32_t *out_len, int32_t *out_path, int32_t max_len, void *stream);

/* ---- diagnostics -------------------------------------------------------- */

/* Counters of the SSSP phase of the last solve (no reference counterpart):
 * whole-graph search: [near-frontier steps, far-list splits, frontier
 * vertices relaxed, far entries scanned, batches], summed over all batches;
 * through the boundary graph (FAP_OPT_SSSP_METHOD): [Bellman-Ford rounds of
 * the local and boundary-graph steps, 0, nodes they visited, 0, 0],
 * summed over their CTAs. */
int fap_sssp_stats(fap_engine *e, uint64_t *out5);

/* Add-min operations per second that the GPU issues from registers alone
 * (no reference counterpart; the roofline denominator of the FW and min-plus
 * phases).  mode 0: int32 DPX add-min (__viaddmin_u32); 1: FP32
 * fminf(a + b, c); 2: int32 add-min keeping the argmin; 3: FP32 add-min
 * keeping the argmin; 4: int32, two add-mins as two adds and one 3-input
 * min; 5: FP32, two add-mins as one paired add (add.f32x2) and one 3-input
 * min; 6-9: FP32 add-min keeping the step of the last strict improvement,
 * as __vibmin_s32 (6), a compare and two predicated moves (7), a float
 * compare, fminf and a select (8), __vibmin_u32 (9); 10: FP32 add-mins in
 * groups of four steps keeping the group of the last strict improvement
 * (a 3-input and a 2-input minimum, a compare, two selects); 11: mode 10
 * with paired adds (add.f32x2); 12: the groups of four as the FP32 strip
 * kernels run them (two 3-input minimums over the current value, a compare,
 * one select). */
int fap_addmin_peak(fap_engine *e, int32_t mode, double *ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* FASTAPSP_H_ */
