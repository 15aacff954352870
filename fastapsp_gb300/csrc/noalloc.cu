// noalloc.cu -- the batched boundary SSSP for callers that cannot allocate
// device memory (no counterpart in the reference).
//
// Some callers of this library must not call cudaMalloc: code that runs while
// a memory pool or an arena owned by someone else is the only allocator
// allowed in the process, plugins whose host framework forbids allocation
// inside a request, or real-time paths where an allocation (and the device
// synchronization it can imply) is not acceptable.  fap_sssp_noalloc gives
// them the SSSP kernel of fap_sssp with every piece of scratch -- the
// per-batch distance table, frontiers, frontier bitmaps, the batch list and
// the status word -- taken from one file-scope device array of fixed size,
// kNoAllocBytes.  The caller passes the graph and the output rows in device
// memory it owns.  Every GPU that loads this library holds the array until
// the process exits.
//
// In host code the array's name is only a host-side stand-in; its device
// address is fetched with cudaGetSymbolAddress once per device (with that
// device current) on the first call there, which also raises the SSSP
// kernels' shared-memory limits on that device.  That first call should
// therefore come before any stream capture.  All calls on a device share the array and
// it keeps the last call's contents, so every call clears the parts that
// must start at zero (the status words; the kernel clears its own tables);
// calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the array and must be
// serialized by the caller.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fap_internal.h"
#include "kernels.cuh"
#include "launch.h"

namespace {

constexpr size_t kNoAllocBytes = FAP_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int scratch_address(int dev, unsigned char **out, int *sms) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fapi::set_error(FAP_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    int count = 0;
    e = cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
      return fapi::set_error(FAP_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
    // The SSSP kernels need more dynamic shared memory than the 48 KiB
    // default; raise their limits on this device here, since a caller of
    // this entry point may never have created an engine (which does the same).
    // Setting a function attribute allocates nothing.
    e = fapk::init_sssp_kernels();
    if (e != cudaSuccess)
      return fapi::set_error(FAP_ERR_CUDA, std::string("SSSP kernel attributes: ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<unsigned char *>(p);
    g_sms[dev] = count;
  }
  *out = g_addr[dev];
  *sms = g_sms[dev];
  return FAP_OK;
}

}  // namespace

extern "C" int fap_sssp_noalloc(int32_t dtype, int32_t n, int64_t m, const int32_t *row_offset,
                                const int32_t *col_val, const void *weight,
                                const int32_t *in_row_offset, const int32_t *in_col_val,
                                const void *in_weight, const int32_t *sources, int32_t num_sources,
                                void *dist, int32_t *pred, int64_t ld, void *stream) {
  using fapi::set_error;
  if (dtype != FAP_DTYPE_F32 && dtype != FAP_DTYPE_I32)
    return set_error(FAP_ERR_INVALID, "fap_sssp_noalloc: unknown dtype");
  if (n < 1 || m < 0 || num_sources < 0 || ld < n || !row_offset || (m > 0 && (!col_val || !weight)))
    return set_error(FAP_ERR_INVALID, "fap_sssp_noalloc: bad graph arguments");
  if (num_sources > 0 && (!sources || !dist))
    return set_error(FAP_ERR_INVALID, "fap_sssp_noalloc: bad source/output arguments");
  if (pred && (!in_row_offset || (m > 0 && (!in_col_val || !in_weight))))
    return set_error(FAP_ERR_INVALID, "fap_sssp_noalloc: predecessors need the in-edge CSR");
  for (int32_t i = 0; i < num_sources; i++)
    if (sources[i] < 0 || sources[i] >= n)
      return set_error(FAP_ERR_INVALID, "fap_sssp_noalloc: source out of range");
  if (num_sources == 0) return FAP_OK;

  // Layout of the static array: status words | batch list | frontier bitmaps
  // (slots x sssp_bits_bytes(n), none when they fit in shared memory) |
  // per-slot scratch (slots x sssp_slot_bytes(n)).
  const int nb = (num_sources + 31) / 32;
  const size_t o_status = 0;
  const size_t o_batches = 256;
  const size_t batch_bytes = round_up((size_t)nb * sizeof(fapk::SsspBatch), 256);
  const size_t o_bits = o_batches + batch_bytes;
  const size_t per_slot = fapk::sssp_slot_bytes(n) + round_up(fapk::sssp_bits_bytes(n), 256);
  if (o_bits + per_slot > kNoAllocBytes)
    return set_error(FAP_ERR_RANGE,
                     "fap_sssp_noalloc: n = " + std::to_string(n) + " with " +
                         std::to_string(num_sources) + " sources needs more than the " +
                         std::to_string(kNoAllocBytes >> 20) + " MiB static scratch");
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return set_error(FAP_ERR_NO_DEVICE, "fap_sssp_noalloc: no current CUDA device");
  unsigned char *base = nullptr;
  int sms = 0;
  int rc = scratch_address(dev, &base, &sms);
  if (rc != FAP_OK) return rc;
  // Largest slot count (one CTA per slot, at most two per SM) that fits.
  auto end_of = [&](size_t k) {
    return o_bits + round_up(k * fapk::sssp_bits_bytes(n), 256) + k * fapk::sssp_slot_bytes(n);
  };
  int slots = std::min(nb, std::max(1, 2 * sms));
  while (slots > 1 && end_of((size_t)slots) > kNoAllocBytes) slots--;
  if (end_of((size_t)slots) > kNoAllocBytes)
    return set_error(FAP_ERR_RANGE, "fap_sssp_noalloc: graph too large for the static scratch");
  const size_t o_slots = o_bits + round_up((size_t)slots * fapk::sssp_bits_bytes(n), 256);

  std::vector<fapk::SsspBatch> batches(nb);
  for (int b = 0; b < nb; b++) {
    fapk::SsspBatch &sb = batches[b];
    std::memset(&sb, 0, sizeof(sb));
    sb.count = std::min(32, num_sources - 32 * b);
    for (int l = 0; l < sb.count; l++) {
      sb.src[l] = sources[32 * b + l];
      sb.row_off[l] = (int64_t)(32 * b + l) * ld;
    }
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Clear what must start at zero: the status words (the kernel clears its
  // own distance tables and bitmaps at the start of every batch).
  if ((ce = cudaMemsetAsync(base + o_status, 0, 256, st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(base + o_batches, batches.data(), (size_t)nb * sizeof(fapk::SsspBatch),
                            cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return set_error(FAP_ERR_CUDA, std::string("fap_sssp_noalloc: ") + cudaGetErrorString(ce));
  fapk::SsspArgs sa{};
  sa.n = n;
  sa.ro = row_offset;
  sa.col = col_val;
  sa.w = weight;
  sa.iro = in_row_offset;
  sa.icol = in_col_val;
  sa.iw = in_weight;
  sa.batches = reinterpret_cast<const fapk::SsspBatch *>(base + o_batches);
  sa.nbatches = nb;
  sa.dist = dist;
  sa.pred = pred;
  sa.scratch = base + o_slots;
  sa.slots = slots;
  sa.bits = base + o_bits;
  sa.status = reinterpret_cast<unsigned *>(base + o_status);
  sa.maxd = nullptr;
  sa.iter_cap = 8 * n + 64;
  sa.lanes = 32;
  sa.acc64 = 0;
  sa.delta = fapk::kSsspNoDelta;
  if ((ce = fapk::launch_sssp(dtype == FAP_DTYPE_F32, sa, st)) != cudaSuccess)
    return set_error(FAP_ERR_CUDA, std::string("fap_sssp_noalloc: ") + cudaGetErrorString(ce));
  unsigned status = 0;
  if ((ce = cudaMemcpyAsync(&status, base + o_status, sizeof(status), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (ce = cudaStreamSynchronize(st)) != cudaSuccess)
    return set_error(FAP_ERR_CUDA, std::string("fap_sssp_noalloc: ") + cudaGetErrorString(ce));
  if (status & fapk::kErrSsspCap) return set_error(FAP_ERR_NOT_CONVERGED, "SSSP reached its iteration cap");
  if (status) return set_error(FAP_ERR_INVALID, "fap_sssp_noalloc: a kernel saw an out-of-range index");
  return FAP_OK;
}
