// fap/fap.h -- drop-in C++ API of the GB300 Fast-APSP engine.
//
// Same class, namespace and member functions as the reference's
// fap::fapGraph (fap/fap.h:23-163 of TomerHaham/FastAPSP), so code written
// against the reference compiles against this header.  The work is done by the
// CUDA engine behind the C ABI in fastapsp.h; this class owns the host-side
// vectors the reference exposes and forwards every solve to the engine.
//
// Differences from the reference, all deliberate:
//  * The metadata constructor (num_vertexs, num_edges, row_offset, col_val,
//    weight, K) is implemented (empty in the reference, fap/fap.cpp:94-98).
//  * A 4-argument file constructor (file, directed, weighted, K) as shown in
//    the reference's README is provided next to the 7-argument one.
//  * The partitioner names "metis", "KaHIP*" and "jet" all select the engine's
//    own multilevel partitioner; any other name throws std::invalid_argument
//    as the reference does (fap/utils/readIdFile.h:287-290).
//  * solveSubGraph's "already processed" set is per object, not a function
//    static (fap/fap.cpp:522), and there is no static shared between objects.
//  * Errors never exit(): solve()/solveSubGraph() return the negative engine
//    status, and constructors throw std::runtime_error.
//  * getDistanceP2P / getPathP2P take (source, target) overloads; the
//    reference's argument-less versions have no body (fap/fap.cpp:674-680).
#ifndef FAP_FAP_H_
#define FAP_FAP_H_

#include <chrono>
#include <cstdint>
#include <set>
#include <string>
#include <vector>

struct fap_engine;

namespace fap {

class fapGraph {
 protected:
  std::string input_graph;
  std::string partitioner;
  const int32_t max_vertexs_num_limit = 20000;  // split threshold (fap/fap.h:35)
  bool is_split = false;
  bool is_path_needed = false;
  bool version = false;
  double time_partitioning = 0;
  double time_sssp = 0;
  double time_floyd = 0;
  double time_min_plus = 0;
  double time_data_transformation = 0;
  double edge_cut = 0;
  double mem_cons_sssp = 0;
  double mem_cons_floyd = 0;
  double mem_cons_min_plus = 0;
  std::vector<float> dist;
  std::vector<int32_t> path;
  int32_t current_subgraph_id = 0;
  std::vector<float> subgraph_dist;
  std::vector<int32_t> subgraph_path;
  int32_t K = 0;
  std::vector<int> graph_id;
  std::vector<int> st2ed;
  std::vector<int> ed2st;
  std::vector<int> C_BlockVer_num;
  std::vector<int> C_BlockVer_offset;
  std::vector<int> C_BlockBdy_num;
  std::vector<int> C_BlockBdy_offset;
  int32_t max_subgraph_vertexs = 0;

 private:
  ::fap_engine *engine_ = nullptr;
  bool int_mode_ = false;
  bool preconditioned_ = false;
  std::set<int32_t> processed_;
  void init_from_csr();
  void ensure_engine();
  void account(bool whole);

 public:
  int32_t num_vertexs = 0;
  int32_t num_edges = 0;
  std::vector<int32_t> adj_size;
  std::vector<int32_t> row_offset;
  std::vector<int32_t> col_val;
  std::vector<float> weight;
  bool directed = false;
  bool weighted = false;

  ~fapGraph();
  fapGraph(const fapGraph &) = delete;
  fapGraph &operator=(const fapGraph &) = delete;

  // Reads graph/<type>/<input_graph>.mtx relative to the working directory
  // (type from directed/weighted, fap/utils/readMatFile.h:43-51) and
  // partitions it into K parts.  `version` selects the solve mode:
  // false = per-part launches, true = all parts batched in a CUDA graph.
  fapGraph(std::string input_graph, bool directed, bool weight, int32_t K,
           std::string partitioner, bool version,
           std::chrono::time_point<std::chrono::high_resolution_clock> &endTimeIo);
  fapGraph(std::string input_graph, bool directed, bool weight, int32_t K);
  fapGraph(int32_t num_vertexs, int64_t num_edges, std::vector<int32_t> row_offset,
           std::vector<int32_t> col_val, std::vector<float> weight, int32_t K);

  void preCondition();
  bool isSplit();
  std::vector<int> getGraphId();

  int32_t solve(bool is_path_needed = false);
  int32_t solveSubGraph(int32_t sub_garph_id, bool is_path_needed = false);

  std::vector<int32_t> getMapping();
  std::vector<float> getAllDistance();
  std::vector<int32_t> getAllPath();
  int32_t getCurrentSubGraphId();
  std::vector<int32_t> getSubGraphIndex(int32_t sub_garph_id);
  std::vector<float> getSubGraphDistance(int32_t sub_garph_id);
  std::vector<int32_t> getSubGraphPath(int32_t sub_garph_id);
  std::vector<float> getDistanceFromOnePoint(int32_t vectex_id);
  std::vector<int32_t> getPathFromOnePoint(int32_t vectex_id);
  float getDistanceP2P();
  std::vector<int32_t> getPathP2P();
  float getDistanceP2P(int32_t source, int32_t target);
  std::vector<int32_t> getPathP2P(int32_t source, int32_t target);
  double getTimeSSSP();
  double getTimeFloyd();
  double getTimeMinPlus();
  double getTimePartitioning();
  double getTimeData();
  int getBoundaryNum();
  int getInnerNum();
  double getMemConsSSSP();
  double getMemConsFloyd();
  double getMemConsMinPlus();
  double getEdgeCut();
  void printResalts();
  bool check_result(float *dist, int *path, int *source, int source_num, int vertexs,
                    int *adj_size, int *row_offset, int *col_val, float *weight,
                    int *graph_id);
};

}  // namespace fap

#endif  // FAP_FAP_H_
