// clm_run_noalloc: pair-map reductions that allocate no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they evaluate energies --
// applications whose device memory is entirely owned by their own pool allocator (a Julia CUDA.jl or
// PyTorch caching pool, an MD engine with a fixed arena: a cudaMalloc behind the pool's back can fail or
// fragment it), and real-time loops that must not call into the CUDA allocator (cudaMalloc and cudaFree
// can block on the whole device).  They build the cell lists once with the ordinary entry points (which
// do allocate), then evaluate scalar reductions of the pair map any number of times through this entry
// point.  The call waits for its result on the handle's stream and reads it on the host.
//
// The per-block partial sums and the final result of the reduction live in one file-scope device array
// of 128 KiB + 256 B (4096 per-block slots), which every GPU that loads this library holds until the
// process exits.  Every call shares it and it keeps the last call's contents; each launched block
// overwrites its own slot and the final reduction overwrites the result, so nothing has to be cleared
// between calls.  Calls that overlap on the GPU (different handles or streams in flight at the same
// time) race on the array: serialize them.
#include <cuda_runtime.h>

#include <mutex>

#include "celllistmap_gb300.h"
#include "clm_internal.hpp"

using namespace clm;

// Same definition as in clm_api.cu: the opaque handle of the C ABI is the library's Handle.
struct clm_handle_s : public Handle {};

namespace {

constexpr size_t kNoAllocScratchBytes = 128 * 1024 + 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// In host code `g_noalloc_scratch` is a host-side stand-in, not a device address: the device address
// is looked up once per device, with that device current, and cached.
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

int scratch_address(clm::Handle& h, void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    h.last_error = "no usable current CUDA device";
    return clm::ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      h.last_error = std::string("cudaGetSymbolAddress failed for the allocation-free scratch: ") +
                     cudaGetErrorString(e);
      return clm::ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return clm::OK;
}

}  // namespace

extern "C" int32_t clm_run_noalloc(clm_handle h, int32_t op_id, const clm_op_params* params, clm_outputs* out) {
  if (!h || !out) return clm::ERR_ARG;
  if (h->batch.on) {
    h->last_error = "a batch handle takes clm_batched_run";
    return clm::ERR_STATE;
  }
  if (!h->box_set) {
    h->last_error = "clm_set_box and clm_build must be called before clm_run_noalloc";
    return clm::ERR_STATE;
  }
  for (int s = 0; s < h->nsets; s++) {
    if (h->sets[s].pending) {
      // a build enqueued by a clm_run that returned early: its totals and error bits were never checked
      h->sets[s].pending = false;
      h->sets[s].dirty = true;
    }
    if (h->sets[s].dirty || !h->sets[s].built) {
      h->last_error = "clm_run_noalloc does not build cell lists (building allocates): call clm_build first";
      return clm::ERR_STATE;
    }
  }
  void* scratch = nullptr;
  int st = scratch_address(*h, &scratch);
  if (st) return st;
  CLM_CUDA_TRY(*h, cudaMemsetAsync(h->err.p, 0, 64, h->stream));
  if (h->dtype == CLM_F64)
    return clm::run_pairs_scalar_scratch<double>(*h, h->gd, op_id, params, out, scratch, kNoAllocScratchBytes);
  return clm::run_pairs_scalar_scratch<float>(*h, h->gf, op_id, params, out, scratch, kNoAllocScratchBytes);
}
