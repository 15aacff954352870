// ref_shim_part.h -- stands in for the reference's partitioner front end when
// the reference's fap.cpp is compiled as a test oracle (oracle/Makefile, `ref`).
//
// TEST INFRASTRUCTURE ONLY.  The reference's readIdFile.h needs METIS, KaHIP,
// Kokkos and Jet headers that are not available, so the build pre-defines its
// include guard and force-includes this file instead.  It supplies
// fap::readIdFile_METIS with the signature of readIdFile.h:293-296 and fills
// the part ids (1-based) and per-part vertex lists (readIdFile.h:279-283) from
// a partition file written by the engine's own partitioner, so both sides run
// on the same partition.  File: n little-endian int32 part ids in 1..K; its
// path is taken from the environment variable FAP_REF_PARTITION.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <string>
#include <unordered_map>
#include <vector>

namespace fap {
inline void readIdFile_METIS(int *id,
                             std::unordered_map<int, std::vector<int>> &BlockVer,
                             int K, bool directed, int vertexs, int edges,
                             int *adj_size, int *row_offset, int *col_val,
                             float *weight, std::string partitioner,
                             double &time_partitioning, double &edge_cut) {
  (void)K; (void)directed; (void)edges; (void)adj_size; (void)row_offset;
  (void)col_val; (void)weight; (void)partitioner;
  const char *p = std::getenv("FAP_REF_PARTITION");
  if (!p) { std::fprintf(stderr, "FAP_REF_PARTITION not set\n"); std::exit(2); }
  FILE *f = std::fopen(p, "rb");
  if (!f) { std::fprintf(stderr, "cannot open %s\n", p); std::exit(2); }
  std::vector<int> part(vertexs);
  size_t got = std::fread(part.data(), sizeof(int), vertexs, f);
  std::fclose(f);
  if (got != (size_t)vertexs) { std::fprintf(stderr, "short partition file\n"); std::exit(2); }
  for (int i = 0; i < vertexs; i++) {
    id[i] = part[i];
    BlockVer[part[i]].push_back(i);
  }
  time_partitioning = 0.0;
  edge_cut = 0.0;
}
}  // namespace fap
