// gbxtb_singlepoint_noalloc: the single point for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc at the time they
// compute.  Examples: a host framework whose memory pool must not grow once
// it is set up, a real-time loop that forbids allocation after start-up, or
// a plugin callback that is handed only a stream.  This entry point takes its
// scratch from a fixed device array compiled into the library instead of a
// caller workspace, and calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// The array (GBXTB_NOALLOC_SCRATCH_BYTES) is a file-scope __device__
// variable.  In host code its name is only a host-side stand-in, not a
// device address, so its device address is looked up with
// cudaGetSymbolAddress once per device, with that device current, by the
// first call made on that device.  Under CUDA's lazy module loading (the
// default) that first lookup is also what loads this file's module onto the
// device, so the array occupies device memory from the first call on a
// device until the process exits; make that first call at set-up, before
// any stream capture.  The cached address does not survive cudaDeviceReset.
// The first call on a plan, and the first after the options or the scratch
// address changed (a gbxtb_singlepoint call with a workspace in between),
// also creates the plan's capture stream and instantiates its pass graphs,
// which is driver work that can take device memory; a warm-up call at
// set-up does it once.  All calls share the one array and it keeps the
// previous call's contents (the single-point driver clears every buffer it
// reads before use); calls whose GPU work overlaps race on it.
#include "internal.cuh"

#include <mutex>
#include <string>

namespace {

constexpr size_t kNoAllocScratchBytes = GBXTB_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

}  // namespace

extern "C" int gbxtb_singlepoint_noalloc(gbxtb_plan *plan, const gbxtb_options *opts,
                                         const double *positions_dev, double *energy_dev,
                                         double *charges_dev, double *gradient_dev, void *stream) {
  if (!plan || !opts) return gbxtb::set_error(GBXTB_ERR_ARG, "null argument");
  if (opts->profile)
    return gbxtb::set_error(GBXTB_ERR_ARG,
                            "profiling creates CUDA events, which gbxtb_singlepoint_noalloc does not do");
  const size_t need = gbxtb::plan_workspace_bytes(plan);
  if (need > kNoAllocScratchBytes)
    return gbxtb::set_error(GBXTB_ERR_WORKSPACE,
                            "plan needs " + std::to_string(need) + " bytes of scratch, more than the " +
                                std::to_string(kNoAllocScratchBytes) +
                                " bytes of gbxtb_singlepoint_noalloc; use gbxtb_singlepoint with a workspace");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return gbxtb::set_error(GBXTB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return gbxtb::set_error(GBXTB_ERR_ARG, "device ordinal out of range");
  // the scratch is the current device's array; the plan's buffers must be
  // on the same device
  if (dev != gbxtb::plan_device(plan))
    return gbxtb::set_error(GBXTB_ERR_ARG, "the current device (" + std::to_string(dev) +
                                               ") is not the device of the plan (" +
                                               std::to_string(gbxtb::plan_device(plan)) + ")");
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return gbxtb::set_error(GBXTB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    scratch = g_scratch_addr[dev];
  }
  return gbxtb_singlepoint(plan, opts, positions_dev, energy_dev, charges_dev, gradient_dev, scratch,
                           kNoAllocScratchBytes, stream);
}
