// fap_more_task.cpp -- the multi-GPU task layer of the drop-in API (see
// include/fap/fap_more_task.h; reference: fap/fap_more_task_mpi.cpp).

#include "fap/fap_more_task.h"

#include <algorithm>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <thread>
#include <utility>

#include "fastapsp.h"

namespace fap {

void fapGraphMoreTask::init(int32_t num_process, int32_t K) {
  if (num_process < 1) throw std::invalid_argument("fapGraphMoreTask::init: num_process < 1");
  this->num_process = num_process;
  tasks_array.assign(K, 0);
  tasks_num.assign(num_process, 0);
  tasks_offset.assign(num_process, 0);
  task_per_process.clear();
}

void fapGraphMoreTask::loadBalance(int32_t num_process) {
  if (tasks_num.size() != (size_t)num_process) init(num_process, K);
  if ((int32_t)C_BlockVer_num.size() < K + 1) preCondition();
  // estimated cost of each part: FW + min-plus + SSSP rows
  std::vector<double> cost(K);
  for (int p = 1; p <= K; p++) {
    const double sub = C_BlockVer_num[p], bdy = C_BlockBdy_num[p];
    cost[p - 1] = sub * sub * sub + (sub - bdy) * num_vertexs * bdy +
                  bdy * ((double)num_vertexs + num_edges);
  }
  std::vector<int> order(K);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  using Load = std::pair<double, int>;  // (load, process): least loaded, then lowest id
  std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
  for (int r = 0; r < num_process; r++) heap.push({0.0, r});
  std::vector<std::vector<int>> per(num_process);
  for (int i : order) {
    Load l = heap.top();
    heap.pop();
    per[l.second].push_back(i + 1);
    heap.push({l.first + cost[i], l.second});
  }
  task_per_process.clear();
  int32_t off = 0;
  for (int r = 0; r < num_process; r++) {
    std::sort(per[r].begin(), per[r].end());
    tasks_offset[r] = off;
    tasks_num[r] = (int32_t)per[r].size();
    for (int p : per[r]) tasks_array[off++] = p;
    task_per_process[r] = per[r];
  }
}

void fapGraphMoreTask::Meta_Bcast(
    const std::function<void(void *data, int64_t count, bool is_float)> &bcast) {
  bcast(adj_size.data(), (int64_t)adj_size.size(), false);
  bcast(row_offset.data(), (int64_t)row_offset.size(), false);
  bcast(col_val.data(), (int64_t)col_val.size(), false);
  bcast(weight.data(), (int64_t)weight.size(), true);
  bcast(st2ed.data(), (int64_t)st2ed.size(), false);
  bcast(ed2st.data(), (int64_t)ed2st.size(), false);
  bcast(graph_id.data(), (int64_t)graph_id.size(), false);
  bcast(C_BlockVer_num.data(), (int64_t)C_BlockVer_num.size(), false);
  bcast(C_BlockVer_offset.data(), (int64_t)C_BlockVer_offset.size(), false);
  bcast(C_BlockBdy_num.data(), (int64_t)C_BlockBdy_num.size(), false);
  bcast(C_BlockBdy_offset.data(), (int64_t)C_BlockBdy_offset.size(), false);
  bcast(tasks_array.data(), (int64_t)tasks_array.size(), false);
  bcast(tasks_num.data(), (int64_t)tasks_num.size(), false);
  bcast(tasks_offset.data(), (int64_t)tasks_offset.size(), false);
  task_per_process.clear();
  for (int r = 0; r < num_process; r++) task_per_process[r] = getCurrentTask(r);
}

std::vector<int> fapGraphMoreTask::getCurrentTask(int32_t process_id) {
  if (process_id < 0 || process_id >= (int32_t)tasks_num.size())
    throw std::out_of_range("fapGraphMoreTask::getCurrentTask: no such process");
  std::vector<int> cur;
  for (int i = 0; i < tasks_num[process_id]; i++) cur.push_back(tasks_array[tasks_offset[process_id] + i]);
  return cur;
}

int32_t fapGraphMoreTask::solveTasks(const std::vector<int32_t> &devices, bool is_path_needed) {
  if ((int32_t)devices.size() != num_process || num_process == 0)
    throw std::invalid_argument("fapGraphMoreTask::solveTasks: one device per process");
  if ((int32_t)C_BlockVer_num.size() < K + 1) preCondition();
  const int64_t n = num_vertexs;
  dist.assign((size_t)(n * n), 0.0f);
  if (is_path_needed) path.assign((size_t)(n * n), -1);
  std::vector<int32_t> status(num_process, FAP_OK);
  std::vector<std::thread> threads;
  for (int r = 0; r < num_process; r++) {
    threads.emplace_back([&, r]() {
      fap_engine *e = nullptr;
      int rc = fap_create(num_vertexs, num_edges, row_offset.data(), col_val.data(), weight.data(),
                          K, graph_id.data(), FAP_DTYPE_F32, devices[r], &e);
      for (int p : getCurrentTask(r)) {
        if (rc != FAP_OK) break;
        const int64_t off = (int64_t)C_BlockVer_offset[p] * n;
        rc = fap_solve_part(e, p, dist.data() + off, is_path_needed ? path.data() + off : nullptr,
                            nullptr);
      }
      if (e) fap_destroy(e);
      status[r] = rc;
    });
  }
  for (auto &t : threads) t.join();
  for (int32_t s : status)
    if (s != FAP_OK) return s;
  return 0;
}

}  // namespace fap
