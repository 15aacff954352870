// ref_main.cpp -- driver for the reference's own fapGraph compiled as a test
// oracle (oracle/Makefile, target `ref`).  TEST INFRASTRUCTURE ONLY.
//
// Usage: fap_ref <workdir> <name> <directed 0/1> <weighted 0/1> <K> <outdir>
//                [part ids ...]
// Reads <workdir>/graph/<type>/<name>.mtx exactly as the reference does
// (readMatFile.h:73-81), partitions with the file in $FAP_REF_PARTITION,
// calls preCondition() and then solve() (no part ids given) or
// solveSubGraph(i) for each given id.  Writes into <outdir>:
//   mapping.i32            getMapping()             (fap.cpp:546-548)
//   dist.f32 / path.i32    getAllDistance/Path      (fap.cpp:550-558), or
//   dist_<i>.f32 / path_<i>.i32 / index_<i>.i32 per solved part
//                          (getSubGraphDistance/Path/Index, fap.cpp:560-580)
//   times.txt              getTime* (fap.cpp:622-639)
#include <unistd.h>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "fap/fap.h"

template <typename T>
static void dump(const std::string &path, const std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(3); }
  std::fwrite(v.data(), sizeof(T), v.size(), f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: %s workdir name directed weighted K outdir [ids]\n", argv[0]);
    return 2;
  }
  std::string workdir = argv[1], name = argv[2], outdir = argv[6];
  bool directed = std::atoi(argv[3]) != 0, weighted = std::atoi(argv[4]) != 0;
  int K = std::atoi(argv[5]);
  if (chdir(workdir.c_str()) != 0) { std::perror("chdir"); return 2; }
  std::chrono::time_point<std::chrono::high_resolution_clock> end_io;
  auto t0 = std::chrono::high_resolution_clock::now();
  fap::fapGraph G(name, directed, weighted, K, "metis", false, end_io);
  G.preCondition();
  dump(outdir + "/mapping.i32", G.getMapping());
  if (argc == 7) {
    G.solve();
    dump(outdir + "/dist.f32", G.getAllDistance());
    dump(outdir + "/path.i32", G.getAllPath());
  } else {
    for (int a = 7; a < argc; a++) {
      int id = std::atoi(argv[a]);
      G.solveSubGraph(id);
      std::string s = std::to_string(id);
      dump(outdir + "/dist_" + s + ".f32", G.getSubGraphDistance(id));
      dump(outdir + "/path_" + s + ".i32", G.getSubGraphPath(id));
      dump(outdir + "/index_" + s + ".i32", G.getSubGraphIndex(id));
    }
  }
  auto t1 = std::chrono::high_resolution_clock::now();
  FILE *f = std::fopen((outdir + "/times.txt").c_str(), "w");
  std::fprintf(f, "total %.6f\nsssp %.6f\nfloyd %.6f\nmin_plus %.6f\ndata %.6f\n",
               std::chrono::duration<double>(t1 - t0).count(), G.getTimeSSSP(),
               G.getTimeFloyd(), G.getTimeMinPlus(), G.getTimeData());
  std::fclose(f);
  return 0;
}
