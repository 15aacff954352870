// fap_graph.cpp -- the drop-in fap::fapGraph class (include/fap/fap.h) over
// the engine's C ABI.  Host-side only: every solve is forwarded to the CUDA
// engine; this file owns the host vectors the reference's class exposes.
// Reference: fap/fap.h:25-162, fap/fap.cpp:45-688.

#include "../../include/fap/fap.h"

#include <sys/time.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <functional>
#include <memory>
#include <queue>
#include <stdexcept>
#include <utility>

#include "../../include/fastapsp.h"

namespace fap {

namespace {

const float kMaxValue = FAP_MAXVALUE_F32;

std::string graph_path(const std::string &name, bool directed, bool weighted) {
  // fap/utils/readMatFile.h:43-51
  std::string type = directed ? (weighted ? "weight-directed" : "unweight-directed")
                              : (weighted ? "weight-undirected" : "unweight-undirected");
  return "graph/" + type + "/" + name + ".mtx";
}

void check(int rc, const char *what) {
  if (rc != FAP_OK)
    throw std::runtime_error(std::string(what) + ": " + fap_status_string(rc) + " (" +
                             fap_last_error() + ")");
}

bool known_partitioner(const std::string &p) {
  // names accepted by the reference's Graph_decomposition (readIdFile.h:84-283)
  return p == "metis" || p == "jet" || p == "KaHIP" || p == "KaHIP_eco" ||
         p == "KaHIP_soc_eco" || p == "KaHIP_soc_s" || p == "KaHIP_soc_f" || p == "KaHIP_f";
}

// Converts int32 results (INF = 2^30) in place to the reference's float
// convention (unreached = 1e8).
void int_to_float_inplace(float *buf, size_t count) {
  int32_t *ib = reinterpret_cast<int32_t *>(buf);
  for (size_t i = 0; i < count; i++) {
    int32_t v = ib[i];
    buf[i] = v >= FAP_INF_I32 ? kMaxValue : (float)v;
  }
}

// Dijkstra used by check_result (the reference's fap::dijkstra,
// fap/kernel/batch_sssp.h:45-77).
void host_dijkstra(int u, int n, const int *row_offset, const int *col_val, const float *w,
                   std::vector<float> &dist) {
  dist.assign(n, kMaxValue);
  dist[u] = 0;
  std::vector<bool> st(n, false);
  typedef std::pair<float, int> PDI;
  std::priority_queue<PDI, std::vector<PDI>, std::greater<PDI>> q;
  q.push({0.0f, u});
  while (!q.empty()) {
    PDI x = q.top();
    q.pop();
    if (st[x.second]) continue;
    st[x.second] = true;
    for (int e = row_offset[x.second]; e < row_offset[x.second + 1]; e++) {
      float c = x.first + w[e];
      if (dist[col_val[e]] > c) {
        dist[col_val[e]] = c;
        q.push({c, col_val[e]});
      }
    }
  }
}

}  // namespace

fapGraph::~fapGraph() {
  if (engine_) fap_destroy(engine_);
  engine_ = nullptr;
}

fapGraph::fapGraph(std::string input_graph, bool directed, bool weighted, int32_t K,
                   std::string partitioner, bool version,
                   std::chrono::time_point<std::chrono::high_resolution_clock> &endTimeIo) {
  if (!known_partitioner(partitioner)) throw std::invalid_argument("Invalid partitioner type");
  this->input_graph = input_graph;
  this->partitioner = partitioner;
  this->directed = directed;
  this->weighted = weighted;
  this->K = K;
  this->version = version;
  const std::string path = graph_path(input_graph, directed, weighted);
  int32_t n = 0;
  int64_t m = 0;
  check(fap_mtx_counts(path.c_str(), directed, weighted, &n, &m), "fap_mtx_counts");
  adj_size.assign(n, 0);
  row_offset.assign((size_t)n + 1, 0);
  col_val.assign((size_t)m, 0);
  weight.assign((size_t)m, 0.0f);
  check(fap_mtx_read(path.c_str(), directed, weighted, n, m, adj_size.data(), row_offset.data(),
                     col_val.data(), weight.data()),
        "fap_mtx_read");
  col_val.resize(row_offset[n]);
  weight.resize(row_offset[n]);
  num_vertexs = n;
  num_edges = row_offset[n];
  endTimeIo = std::chrono::high_resolution_clock::now();
  init_from_csr();
}

fapGraph::fapGraph(std::string input_graph, bool directed, bool weighted, int32_t K)
    : fapGraph(input_graph, directed, weighted, K, "metis", false,
               *std::make_unique<std::chrono::time_point<std::chrono::high_resolution_clock>>()) {}

fapGraph::fapGraph(int32_t num_vertexs, int64_t num_edges, std::vector<int32_t> row_offset,
                   std::vector<int32_t> col_val, std::vector<float> weight, int32_t K) {
  if (num_vertexs < 0 || (int64_t)row_offset.size() != (int64_t)num_vertexs + 1 ||
      (int64_t)col_val.size() != num_edges || (int64_t)weight.size() != num_edges)
    throw std::invalid_argument("fapGraph: CSR sizes do not match num_vertexs/num_edges");
  this->num_vertexs = num_vertexs;
  this->num_edges = (int32_t)num_edges;
  this->row_offset = std::move(row_offset);
  this->col_val = std::move(col_val);
  this->weight = std::move(weight);
  this->K = K;
  this->partitioner = "metis";
  this->directed = true;
  this->weighted = true;
  adj_size.resize(num_vertexs);
  for (int32_t i = 0; i < num_vertexs; i++) adj_size[i] = this->row_offset[i + 1] - this->row_offset[i];
  init_from_csr();
}

void fapGraph::init_from_csr() {
  graph_id.assign(num_vertexs, 0);
  st2ed.assign(num_vertexs, 0);
  ed2st.assign(num_vertexs, 0);
  C_BlockVer_num.assign(K + 1, 0);
  C_BlockVer_offset.assign(K + 1, 0);
  C_BlockBdy_num.assign(K + 1, 0);
  C_BlockBdy_offset.assign(K + 1, 0);
  auto t0 = std::chrono::high_resolution_clock::now();
  int64_t cut = 0;
  check(fap_partition(num_vertexs, row_offset.data(), col_val.data(), K, 1, graph_id.data(), &cut),
        "fap_partition");
  time_partitioning =
      std::chrono::duration<double>(std::chrono::high_resolution_clock::now() - t0).count();
  edge_cut = (double)cut;
  // Integer weights whose sums stay exact in FP32 are solved in int32 mode;
  // the results are converted to the reference's float convention.
  float wmax = 0;
  bool integer = true;
  for (float w : weight) {
    integer = integer && w == std::floor(w) && w >= 0;
    wmax = std::max(wmax, w);
  }
  int_mode_ = integer && (double)wmax * std::max(num_vertexs - 1, 1) < (double)(1 << 24);
}

void fapGraph::preCondition() {
  check(fap_preprocess(K, num_vertexs, graph_id.data(), row_offset.data(), col_val.data(),
                       st2ed.data(), ed2st.data(), C_BlockVer_num.data(), C_BlockVer_offset.data(),
                       C_BlockBdy_num.data(), C_BlockBdy_offset.data()),
        "fap_preprocess");
  max_subgraph_vertexs = 0;
  for (int i = 1; i <= K; i++) max_subgraph_vertexs = std::max(max_subgraph_vertexs, C_BlockVer_num[i]);
  is_split = num_vertexs > max_vertexs_num_limit;
  preconditioned_ = true;
}

void fapGraph::ensure_engine() {
  if (!preconditioned_) preCondition();
  if (engine_) return;
  int dev = 0;
  if (const char *d = std::getenv("FAP_DEVICE")) dev = std::atoi(d);
  check(fap_create(num_vertexs, row_offset[num_vertexs], row_offset.data(), col_val.data(),
                   weight.data(), K, graph_id.data(), int_mode_ ? FAP_DTYPE_I32 : FAP_DTYPE_F32,
                   dev, &engine_),
        "fap_create");
}

bool fapGraph::isSplit() { return is_split; }

std::vector<int> fapGraph::getGraphId() { return graph_id; }

void fapGraph::account(bool whole) {
  double t[5];
  if (fap_last_times(engine_, t) != FAP_OK) return;
  time_sssp += t[0] / 1e3;
  time_floyd += t[1] / 1e3;
  time_min_plus += t[2] / 1e3;
  time_data_transformation += t[3] / 1e3;
  (void)whole;
}

int32_t fapGraph::solve(bool is_path_needed) {
  this->is_path_needed = is_path_needed;
  ensure_engine();
  const size_t total = (size_t)num_vertexs * num_vertexs;
  dist.resize(total);
  path.resize(total);
  int rc = fap_solve(engine_, dist.data(), path.data(),
                     version ? FAP_MODE_BATCHED : FAP_MODE_PLAIN, nullptr);
  if (rc != FAP_OK) return rc;
  if (int_mode_) int_to_float_inplace(dist.data(), total);
  account(true);
  return 0;
}

int32_t fapGraph::solveSubGraph(int32_t sub_graph_id, bool is_path_needed) {
  this->is_path_needed = is_path_needed;
  if (processed_.count(sub_graph_id)) {
    std::printf("Warning: Subgraph %d has already been processed, skipping.\n", sub_graph_id);
    return 0;
  }
  ensure_engine();
  if (sub_graph_id < 1 || sub_graph_id > K) return FAP_ERR_INVALID;
  const size_t total = (size_t)C_BlockVer_num[sub_graph_id] * num_vertexs;
  subgraph_dist.resize(total);
  subgraph_path.resize(total);
  current_subgraph_id = sub_graph_id;
  processed_.insert(sub_graph_id);
  int rc = fap_solve_part(engine_, sub_graph_id, subgraph_dist.data(), subgraph_path.data(), nullptr);
  if (rc != FAP_OK) return rc;
  if (int_mode_) int_to_float_inplace(subgraph_dist.data(), total);
  account(false);
  return 0;
}

std::vector<int32_t> fapGraph::getMapping() { return st2ed; }

std::vector<float> fapGraph::getAllDistance() {
  if (is_split) throw std::logic_error("getAllDistance: graph is split; use solveSubGraph");
  return dist;
}

std::vector<int32_t> fapGraph::getAllPath() {
  if (is_split) throw std::logic_error("getAllPath: graph is split; use solveSubGraph");
  return path;
}

std::vector<int32_t> fapGraph::getSubGraphIndex(int32_t id) {
  int off = C_BlockVer_offset[id], size = C_BlockVer_num[id];
  return std::vector<int32_t>(st2ed.begin() + off, st2ed.begin() + off + size);
}

int32_t fapGraph::getCurrentSubGraphId() { return current_subgraph_id; }

std::vector<float> fapGraph::getSubGraphDistance(int32_t id) {
  if (current_subgraph_id != id) throw std::logic_error("getSubGraphDistance: not the current subgraph");
  return subgraph_dist;
}

std::vector<int32_t> fapGraph::getSubGraphPath(int32_t id) {
  if (current_subgraph_id != id) throw std::logic_error("getSubGraphPath: not the current subgraph");
  return subgraph_path;
}

// Row of `v` in the current subgraph's result (the reference indexes
// C_BlockVer_offset by the vertex id, fap/fap.cpp:584-587; the part's offset
// is what is meant).
std::vector<float> fapGraph::getDistanceFromOnePoint(int32_t v) {
  if (graph_id[v] != current_subgraph_id) throw std::logic_error("vertex not in the current subgraph");
  size_t row = (size_t)(ed2st[v] - C_BlockVer_offset[current_subgraph_id]);
  return std::vector<float>(subgraph_dist.begin() + row * num_vertexs,
                            subgraph_dist.begin() + (row + 1) * num_vertexs);
}

std::vector<int32_t> fapGraph::getPathFromOnePoint(int32_t v) {
  if (graph_id[v] != current_subgraph_id) throw std::logic_error("vertex not in the current subgraph");
  size_t row = (size_t)(ed2st[v] - C_BlockVer_offset[current_subgraph_id]);
  return std::vector<int32_t>(subgraph_path.begin() + row * num_vertexs,
                              subgraph_path.begin() + (row + 1) * num_vertexs);
}

float fapGraph::getDistanceP2P() { return kMaxValue; }
std::vector<int32_t> fapGraph::getPathP2P() { return {}; }

float fapGraph::getDistanceP2P(int32_t s, int32_t t) {
  if (s < 0 || s >= num_vertexs || t < 0 || t >= num_vertexs) throw std::out_of_range("vertex id");
  if (!dist.empty()) return dist[(size_t)ed2st[s] * num_vertexs + t];
  return getDistanceFromOnePoint(s)[t];
}

std::vector<int32_t> fapGraph::getPathP2P(int32_t s, int32_t t) {
  if (s < 0 || s >= num_vertexs || t < 0 || t >= num_vertexs) throw std::out_of_range("vertex id");
  std::vector<int32_t> row;
  if (!path.empty()) {
    row.assign(path.begin() + (size_t)ed2st[s] * num_vertexs,
               path.begin() + (size_t)(ed2st[s] + 1) * num_vertexs);
  } else {
    row = getPathFromOnePoint(s);
  }
  std::vector<int32_t> out;
  int32_t v = t;
  for (int steps = 0; steps <= num_vertexs; steps++) {
    if (v < 0) return {};
    out.push_back(v);
    if (v == s) {
      std::reverse(out.begin(), out.end());
      return out;
    }
    v = row[v];
  }
  return {};
}

void fapGraph::printResalts() {
  for (int32_t i = 0; i < num_vertexs; ++i)
    for (int32_t j = 0; j < num_vertexs; ++j)
      std::printf("Distances from node %d:  to node %d: %.2f \n", i, j,
                  dist[(size_t)num_vertexs * i + j]);
}

double fapGraph::getTimePartitioning() { return time_partitioning; }
double fapGraph::getTimeData() { return time_data_transformation; }
double fapGraph::getTimeFloyd() { return time_floyd; }
double fapGraph::getTimeMinPlus() { return time_min_plus; }
double fapGraph::getTimeSSSP() { return time_sssp; }

int fapGraph::getBoundaryNum() {
  int s = 0;
  for (int v : C_BlockBdy_num) s += v;
  return s;
}

int fapGraph::getInnerNum() {
  int s = 0;
  for (size_t i = 0; i < C_BlockVer_num.size(); i++) s += C_BlockVer_num[i] - C_BlockBdy_num[i];
  return s;
}

double fapGraph::getMemConsSSSP() { return mem_cons_sssp / std::max(K, 1); }
double fapGraph::getMemConsFloyd() { return mem_cons_floyd / std::max(K, 1); }
double fapGraph::getMemConsMinPlus() { return mem_cons_min_plus / std::max(K, 1); }
double fapGraph::getEdgeCut() { return edge_cut; }

// Sampled check against Dijkstra, as the reference's check_ans
// (fap/utils/checkResult.h:38-94): 20 random rows x 10 random columns, pairs
// unreached on both sides skipped.  The tolerance is 1e-5 relative (absolute
// below 1): the reference's absolute 1e-5 is smaller than one FP32 ulp for
// distances above 128, where any change of summation order trips it.
bool fapGraph::check_result(float *dist, int *path, int *source, int source_num, int vertexs,
                            int *adj_size, int *row_offset, int *col_val, float *weight,
                            int *graph_id) {
  (void)path;
  (void)adj_size;
  (void)graph_id;
  if (source_num <= 0 || vertexs <= 0) return true;
  unsigned seed = (unsigned)time(nullptr);
  std::vector<float> ref;
  for (int c = 0; c < 20; c++) {
    int vi = rand_r(&seed) % source_num;
    host_dijkstra(source[vi], vertexs, row_offset, col_val, weight, ref);
    for (int d = 0; d < 10; d++) {
      int des = rand_r(&seed) % vertexs;
      float now = dist[(size_t)vi * vertexs + des];
      if (now > kMaxValue / 10 && ref[des] > kMaxValue / 10) continue;
      if (std::fabs(now - ref[des]) > 1e-5f * std::max(1.0f, std::fabs(ref[des]))) {
        std::printf("the dist is wrong!\n%f - %f \n", ref[des], now);
        return false;
      }
    }
  }
  return true;
}

}  // namespace fap
