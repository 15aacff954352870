/*
 * fap_oracle.h -- CPU oracle for the Fast-APSP hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a CPU restatement of the
 * reference's CPU code path (TomerHaham/FastAPSP, `fapGraph::run` host-buffer
 * branch, fap/fap.cpp:400-502).  It exists to check the CUDA engine and to
 * time the reference's CPU algorithm as a baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product path (libfastapsp) never links or calls it.
 *
 * Parity pin: the restatement is checked bit-for-bit against the reference's
 * own fap.cpp compiled from its sources (oracle/Makefile target `ref`) on the
 * committed golden graphs (tests/golden/).  All arithmetic is FP32 like the
 * reference (fap/fap.h:52), with the unreached sentinel 1e8
 * (fap/utils/parameter.h:26).  An extra FP64 Dijkstra serves as the
 * high-precision oracle for FP32-weighted graphs.
 */
#ifndef FAP_ORACLE_H_
#define FAP_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_MAXVALUE 1e8f

/* MatrixMarket reader with the reference's semantics (readMatFile.h:36-173):
 * 1-based ids, undirected inputs doubled, |w| for weighted inputs, weight 1
 * for unweighted inputs, duplicates and self loops kept, each CSR row in
 * reverse insertion order (linked-list prepend).  `path` is the full file
 * path.  Returns 0 on success, -1 if the file cannot be opened. */
int oracle_mtx_counts(const char *path, int directed, int weighted,
                      int32_t *n, int64_t *m);
int oracle_mtx_read(const char *path, int directed, int weighted,
                    int32_t n, int64_t m, int32_t *adj_size,
                    int32_t *row_offset, int32_t *col_val, float *weight);

/* Single-source Dijkstra with predecessors (batch_sssp.h:79-114). */
void oracle_dijkstra_path(int32_t u, int32_t n, const int32_t *adj_size,
                          const int32_t *row_offset, const int32_t *col_val,
                          const float *weight, float *dist, int32_t *path);
/* FP64 Dijkstra over the same CSR with FP64 weights (distance only,
 * 1e300 = unreached). */
void oracle_dijkstra_f64(int32_t u, int32_t n, const int32_t *row_offset,
                         const int32_t *col_val, const double *weight,
                         double *dist);
/* Batched SSSP over `num` sources, OpenMP over sources like
 * batched_sssp_path (batch_sssp.h:232-252). */
void oracle_batched_sssp_path(const int32_t *sources, int32_t num,
                              int32_t n, const int32_t *adj_size,
                              const int32_t *row_offset,
                              const int32_t *col_val, const float *weight,
                              float *dist, int32_t *path);

/* Naive Floyd-Warshall with predecessors (floyd.h:38-49). */
void oracle_floyd_path(int32_t num, float *mat, int32_t *path);

/* res = mat1 (MxK) (min,+) mat2 (KxN); path = mat2_path of the first k that
 * reaches the minimum (minplus.h:51-65). */
void oracle_min_plus_path_advanced(const float *mat1, const float *mat2,
                                   const int32_t *mat2_path, float *res,
                                   int32_t *path, int32_t M, int32_t N,
                                   int32_t K);

/* findBoundry + sort_and_encode (util_preprocess.h:32-106).  graph_id holds
 * part ids in 1..K.  Outputs st2ed/ed2st (n each) and the four K+1 arrays
 * C_BlockVer_num/offset, C_BlockBdy_num/offset (index 0 unused).  Also fills
 * is_boundary (n, 0/1). */
void oracle_preprocess(int32_t K, int32_t n, const int32_t *graph_id,
                       const int32_t *adj_size, const int32_t *row_offset,
                       const int32_t *col_val, int32_t *st2ed, int32_t *ed2st,
                       int32_t *ver_num, int32_t *ver_offset, int32_t *bdy_num,
                       int32_t *bdy_offset, int32_t *is_boundary);

/* Phase timers of one oracle_run_part call, seconds. */
typedef struct {
  double sssp, floyd, min_plus, data;
} oracle_times;

/* One part of fapGraph::run's host-buffer branch (fap.cpp:400-502): writes
 * the sub x n rows of part `part_id` (1-based) into dist/path, rows in st2ed
 * order, columns by original id.  `mp_rows` < 0 runs the full min-plus;
 * otherwise only the first mp_rows inner rows are computed (a bounded sample
 * for timing; the remaining inner rows are left untouched). */
void oracle_run_part(int32_t part_id, int32_t n, const int32_t *adj_size,
                     const int32_t *row_offset, const int32_t *col_val,
                     const float *weight, const int32_t *graph_id,
                     const int32_t *st2ed, const int32_t *ed2st,
                     const int32_t *ver_num, const int32_t *ver_offset,
                     const int32_t *bdy_num, float *dist, int32_t *path,
                     int32_t mp_rows, oracle_times *times);

/* Number of OpenMP threads the SSSP phase uses (0 = library default). */
void oracle_set_threads(int32_t threads);
int32_t oracle_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* FAP_ORACLE_H_ */
