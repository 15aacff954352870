// fap/fap_more_task.h -- multi-GPU task layer of the drop-in API.
//
// Counterpart of the reference's fapGraphMoreTaskMPI
// (fap/fap_more_task_mpi.h:23-50, fap/fap_more_task_mpi.cpp): the same
// members and the same init / loadBalance / getCurrentTask calls, so a
// caller that distributes parts over processes keeps its structure.  Parts
// are independent once every process holds the CSR and the partition, and no
// result is exchanged, as in the reference.  Differences, all deliberate:
//  * loadBalance is deterministic and cost-balanced (longest processing time
//    first on sub^3 + inner * n * bdy + bdy * (n + m)) instead of a random
//    shuffle into equal counts (fap_more_task_mpi.cpp:39-52);
//  * the metadata broadcast takes the caller's collective (MPI_Bcast, NCCL,
//    torch.distributed, ...) as a callback instead of an MPI communicator, so
//    the library itself has no MPI dependency;
//  * solveTasks runs the tasks of several "processes" as host threads, one
//    engine per GPU, writing each part's rows into the getAllDistance() /
//    getAllPath() layout of this object.
#ifndef FAP_FAP_MORE_TASK_H_
#define FAP_FAP_MORE_TASK_H_

#include <cstdint>
#include <functional>
#include <unordered_map>
#include <vector>

#include "fap/fap.h"

namespace fap {

class fapGraphMoreTask : public fapGraph {
 public:
  // parts (1-based ids) of every process, and the same as flat arrays
  std::unordered_map<int, std::vector<int>> task_per_process;
  std::vector<int32_t> tasks_array;   // part ids, process by process
  std::vector<int32_t> tasks_num;     // parts of each process
  std::vector<int32_t> tasks_offset;  // first entry of each process in tasks_array
  int32_t num_process = 0;

  using fapGraph::fapGraph;

  // Sizes the task arrays (call after preCondition()).
  void init(int32_t num_process, int32_t K);
  // Assigns the K parts to num_process processes.
  void loadBalance(int32_t num_process);
  // Broadcasts the metadata a process needs to solve its parts, array by
  // array, through `bcast(data, count, is_float)` (count elements of int32_t,
  // or of float when is_float).  Receivers must hold arrays of the same sizes
  // (an object built from the same graph and K), as with the reference's
  // Meta_MPI_Bcast (fap_more_task_mpi.cpp:57-79).
  void Meta_Bcast(const std::function<void(void *data, int64_t count, bool is_float)> &bcast);
  // Parts of process `process_id`.
  std::vector<int> getCurrentTask(int32_t process_id);
  // Solves the tasks of process i on GPU devices[i], all processes at once
  // (one host thread each); the rows land in getAllDistance()/getAllPath().
  // Returns 0 or the first negative engine status.
  int32_t solveTasks(const std::vector<int32_t> &devices, bool is_path_needed = false);
};

}  // namespace fap

#endif  // FAP_FAP_MORE_TASK_H_
