// single_node_example.cpp -- command-line driver of the drop-in fap::fapGraph
// with the argument set of the reference's app/singleNodeExample.cpp:40-54:
//   -f <name> -k <K> -direct true|false -weight true|false
//   -partitioner <metis|KaHIP*|jet> -version true|false
// The graph is read from graph/<type>/<name>.mtx in the working directory.
// As in the reference, a graph above 20,000 vertices with K >= 3 solves parts
// 1..3 with solveSubGraph, anything else runs solve(); the last solved part is
// then spot-checked against Dijkstra (check_result).
// Extra option: -dump <dir> writes mapping.i32 and, for solve(), dist.f32 /
// path.i32, or per solved part dist_<i>.f32 / path_<i>.i32 / index_<i>.i32.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fap/fap.h"

template <typename T>
static void dump(const std::string &path, const std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return;
  std::fwrite(v.data(), sizeof(T), v.size(), f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  std::string file, partitioner = "metis", dump_dir;
  int K = 1;
  bool directed = false, weighted = false, version = false;
  for (int i = 1; i + 1 < argc; i++) {
    if (!std::strcmp(argv[i], "-f")) file = argv[i + 1];
    else if (!std::strcmp(argv[i], "-k")) K = std::stoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "-direct")) directed = !std::strcmp(argv[i + 1], "true");
    else if (!std::strcmp(argv[i], "-weight")) weighted = !std::strcmp(argv[i + 1], "true");
    else if (!std::strcmp(argv[i], "-partitioner")) partitioner = argv[i + 1];
    else if (!std::strcmp(argv[i], "-version")) version = !std::strcmp(argv[i + 1], "true");
    else if (!std::strcmp(argv[i], "-dump")) dump_dir = argv[i + 1];
  }
  auto start = std::chrono::high_resolution_clock::now();
  std::chrono::time_point<std::chrono::high_resolution_clock> end_io;
  try {
    fap::fapGraph G(file, directed, weighted, K, partitioner, version, end_io);
    G.preCondition();
    if (!dump_dir.empty()) dump(dump_dir + "/mapping.i32", G.getMapping());
    std::vector<int> solved;
    if (G.isSplit() && K >= 3) {
      for (int id = 1; id <= 3; id++) {
        if (G.solveSubGraph(id, true) != 0) return 1;
        solved.push_back(id);
        if (!dump_dir.empty()) {
          std::string s = std::to_string(id);
          dump(dump_dir + "/dist_" + s + ".f32", G.getSubGraphDistance(id));
          dump(dump_dir + "/path_" + s + ".i32", G.getSubGraphPath(id));
          dump(dump_dir + "/index_" + s + ".i32", G.getSubGraphIndex(id));
        }
      }
    } else {
      if (G.solve() != 0) return 1;
      if (!dump_dir.empty()) {
        dump(dump_dir + "/dist.f32", G.getAllDistance());
        dump(dump_dir + "/path.i32", G.getAllPath());
      }
    }
    double total = std::chrono::duration<double>(std::chrono::high_resolution_clock::now() - start).count();
    std::printf("Total runtime: %f seconds.\n", total);
    std::printf("sssp %.6f floyd %.6f min_plus %.6f data %.6f partition %.6f (s)\n", G.getTimeSSSP(),
                G.getTimeFloyd(), G.getTimeMinPlus(), G.getTimeData(), G.getTimePartitioning());
    // verify the last solved part (or part 1 of a full solve)
    int id = solved.empty() ? 1 : solved.back();
    std::vector<int> source = G.getSubGraphIndex(id);
    std::vector<float> rows;
    std::vector<int> prow;
    if (solved.empty()) {
      std::vector<float> all = G.getAllDistance();
      std::vector<int> allp = G.getAllPath();
      std::vector<int> map = G.getMapping();
      // rows of part `id` sit at its offset in the stacked solve() layout
      size_t off = 0;
      for (int p = 1; p < id; p++) off += G.getSubGraphIndex(p).size();
      rows.assign(all.begin() + off * G.num_vertexs, all.begin() + (off + source.size()) * G.num_vertexs);
      prow.assign(allp.begin() + off * G.num_vertexs, allp.begin() + (off + source.size()) * G.num_vertexs);
    } else {
      rows = G.getSubGraphDistance(id);
      prow = G.getSubGraphPath(id);
    }
    std::vector<int> gid = G.getGraphId();
    bool ok = G.check_result(rows.data(), prow.data(), source.data(), (int)source.size(),
                             G.num_vertexs, G.adj_size.data(), G.row_offset.data(),
                             G.col_val.data(), G.weight.data(), gid.data());
    std::printf(ok ? "the %d subGraph is right\n" : "the %d subGraph is wrong !!!\n", id);
    return ok ? 0 : 3;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 2;
  }
}
