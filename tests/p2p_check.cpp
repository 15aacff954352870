// Point-to-point getters of the drop-in class (fap::fapGraph::getDistanceP2P /
// getPathP2P with (source, target)), built and run by tests/test_gpu_query.py.
// argv: <dir> holding ro.i32, col.i32, w.f32 (a CSR), queries.i32 (pairs);
// argv[2] = K, argv[3] = "split" to query after solveSubGraph of the source's
// part instead of solve().  Prints one line per query:
// "s t distance len v0 v1 ... v_len-1".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "fap/fap.h"

template <typename T>
static std::vector<T> load(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<T> out(raw.size() / sizeof(T));
  std::memcpy(out.data(), raw.data(), out.size() * sizeof(T));
  return out;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const std::string dir = argv[1];
  const int K = std::atoi(argv[2]);
  const bool split = argc > 3 && std::string(argv[3]) == "split";
  std::vector<int32_t> ro = load<int32_t>(dir + "/ro.i32"), col = load<int32_t>(dir + "/col.i32");
  std::vector<float> w = load<float>(dir + "/w.f32");
  std::vector<int32_t> q = load<int32_t>(dir + "/queries.i32");
  const int n = (int)ro.size() - 1;
  fap::fapGraph g(n, (int64_t)col.size(), ro, col, w, K);
  g.preCondition();
  if (!split) g.solve(true);
  std::vector<int> gid = g.getGraphId();
  int cur = -1;
  for (size_t i = 0; i + 1 < q.size(); i += 2) {
    const int s = q[i], t = q[i + 1];
    if (split && gid[s] != cur) {
      cur = gid[s];
      g.solveSubGraph(cur, true);
    }
    const float d = g.getDistanceP2P(s, t);
    const std::vector<int32_t> p = g.getPathP2P(s, t);
    std::printf("%d %d %.9g %zu", s, t, d, p.size());
    for (int32_t v : p) std::printf(" %d", v);
    std::printf("\n");
  }
  return 0;
}
