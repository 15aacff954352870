// Checks of the multi-GPU task layer (fap::fapGraphMoreTask), built and run
// by tests/test_more_task.py.  argv[1] = "cpu": task assignment and metadata
// broadcast only; "gpu": also solveTasks on two engines of GPU 0 against a
// plain fapGraph::solve of the same graph.  Prints "OK" on success.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fap/fap.h"
#include "fap/fap_more_task.h"

static void grid(int R, int Cc, std::vector<int32_t> &ro, std::vector<int32_t> &col,
                 std::vector<float> &w) {
  const int n = R * Cc;
  std::vector<std::vector<std::pair<int, float>>> adj(n);
  for (int r = 0; r < R; r++)
    for (int c = 0; c < Cc; c++) {
      const int v = r * Cc + c;
      const float wt = 1.0f + (float)((r * 7 + c * 3) % 5);
      if (c + 1 < Cc) { adj[v].push_back({v + 1, wt}); adj[v + 1].push_back({v, wt}); }
      if (r + 1 < R) { adj[v].push_back({v + Cc, wt + 1}); adj[v + Cc].push_back({v, wt + 1}); }
    }
  ro.assign(1, 0);
  for (int v = 0; v < n; v++) {
    for (auto &e : adj[v]) { col.push_back(e.first); w.push_back(e.second); }
    ro.push_back((int32_t)col.size());
  }
}

int main(int argc, char **argv) {
  const bool gpu = argc > 1 && std::string(argv[1]) == "gpu";
  std::vector<int32_t> ro, col;
  std::vector<float> w;
  grid(24, 20, ro, col, w);
  const int n = (int)ro.size() - 1, K = 7, P = 3;
  fap::fapGraphMoreTask g(n, (int64_t)col.size(), ro, col, w, K);
  g.preCondition();
  g.init(P, K);
  g.loadBalance(P);
  // every part exactly once, and the flat arrays agree with the map
  std::vector<int> seen(K + 1, 0);
  for (int r = 0; r < P; r++) {
    std::vector<int> t = g.getCurrentTask(r);
    if (t != g.task_per_process[r]) { printf("task map mismatch\n"); return 1; }
    for (int p : t) seen[p]++;
  }
  for (int p = 1; p <= K; p++)
    if (seen[p] != 1) { printf("part %d assigned %d times\n", p, seen[p]); return 1; }
  // broadcast to a second object built from the same graph, through a fake
  // collective that copies the root's arrays in order
  fap::fapGraphMoreTask h(n, (int64_t)col.size(), ro, col, w, K);
  h.preCondition();
  h.init(P, K);
  std::vector<std::vector<char>> sent;
  g.Meta_Bcast([&](void *d, int64_t cnt, bool f) {
    sent.emplace_back((char *)d, (char *)d + cnt * (f ? sizeof(float) : sizeof(int32_t)));
  });
  size_t i = 0;
  h.Meta_Bcast([&](void *d, int64_t cnt, bool f) {
    const size_t bytes = cnt * (f ? sizeof(float) : sizeof(int32_t));
    if (i >= sent.size() || sent[i].size() != bytes) { printf("bcast size mismatch\n"); std::exit(1); }
    std::memcpy(d, sent[i].data(), bytes);
    i++;
  });
  for (int r = 0; r < P; r++)
    if (h.getCurrentTask(r) != g.getCurrentTask(r)) { printf("bcast tasks mismatch\n"); return 1; }
  if (h.getMapping() != g.getMapping()) { printf("bcast mapping mismatch\n"); return 1; }
  if (gpu) {
    if (g.solveTasks({0, 0, 0}, true) != 0) { printf("solveTasks failed\n"); return 1; }
    std::vector<float> d = g.getAllDistance();
    std::vector<int32_t> p = g.getAllPath();
    fap::fapGraph ref(n, (int64_t)col.size(), ro, col, w, K);
    ref.preCondition();
    if (ref.solve(true) != 0) { printf("solve failed\n"); return 1; }
    if (d != ref.getAllDistance()) { printf("distances differ\n"); return 1; }
    std::vector<int32_t> rp = ref.getAllPath();
    if (p != rp) { printf("predecessors differ\n"); return 1; }
  }
  printf("OK\n");
  return 0;
}
