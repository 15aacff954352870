// fap_internal.h -- declarations shared by the engine's translation units.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fastapsp.h"

namespace fapi {

// Records `msg` as this thread's last error and returns `status`.
int set_error(int status, const std::string &msg);
void clear_error();
const char *last_error();

// host_prep.cpp
int mtx_counts(const char *path, bool directed, int32_t *n, int64_t *m);
int mtx_read(const char *path, bool directed, bool weighted, int32_t n, int64_t m,
             int32_t *adj_size, int32_t *row_offset, int32_t *col_val, float *weight);
int partition(int32_t n, const int32_t *ro, const int32_t *col, int32_t K, uint64_t seed,
              int32_t *graph_id, int64_t *edge_cut);
int preprocess(int32_t K, int32_t n, const int32_t *graph_id, const int32_t *ro,
               const int32_t *col, int32_t *st2ed, int32_t *ed2st, int32_t *ver_num,
               int32_t *ver_offset, int32_t *bdy_num, int32_t *bdy_offset,
               std::vector<uint8_t> *is_boundary);

}  // namespace fapi
