// ommp_gpu_tmatvec_noalloc: the T.mu product of a system into caller-owned
// device memory, with no memory allocation of any kind during the call.
//
// Who needs it: host programs that own all GPU memory themselves and cannot
// let a library call cudaMalloc/cudaFree while they run -- for example a
// quantum-chemistry code driving the polarization from inside its own SCF
// loop with a preallocated memory pool, or a molecular-dynamics engine whose
// time step must not stall: cudaMalloc and cudaFree synchronise the device
// and can fail at an arbitrary point of a long run.  The regular entry point
// ommp_gpu_tmatvec stages through the system's own buffers; this variant
// takes device pointers and keeps its only scratch (the fixed-point sums of
// the symmetric product from 2048 sites, else the per-source-split partial
// fields of the target-outer kernel) in a fixed, file-scope device array.
//
// The product is always the direct FP64 sum over all pairs: the system's FMM
// switch, its matrix-vector selector (in-core T) and its FP64 kernel choice
// do not apply here.
//
// The scratch array (kNoAllocScratchBytes = 16 MiB) lives in every GPU that
// loads this library until the process exits.  Its device address is looked
// up with that device current when a system is created on it
// (noalloc_prepare_device, called from the system's device set-up, where
// allocation already happens); that lookup is what makes the CUDA runtime
// load this file's module and place the array.  A call on a device where no
// system was created first does the lookup itself: that first call is then
// set-up and should come before any stream capture.  All calls share the
// array: two calls whose kernels overlap on a GPU (from different host
// threads, or different systems on different streams) race on it.  The call
// itself waits for its kernels, so calls issued one after another from one
// thread never overlap.  What must start at zero is cleared on every call:
// the symmetric branch clears its fixed-point accumulators with
// cudaMemsetAsync before its pair kernel; in the target-outer branch every
// partial the finishing kernel reads is first written by the pair kernel of
// the same call.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/openmmpol_gb300.h"
#include "engine.h"
#include "kernels.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
constexpr size_t kNoAllocScratchDoubles = kNoAllocScratchBytes / sizeof(double);
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the static scratch on the current device (set-up once).
int scratch_address(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return ommp::kErrCuda;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    ommp::set_last_error("device ordinal out of range for the no-allocation scratch table");
    return ommp::kErrBadArg;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      ommp::set_last_error(std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(e));
      return ommp::kErrCuda;
    }
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return ommp::kOk;
}

bool ranges_overlap(const void *a, const void *b, size_t bytes) {
  const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
  return pa < pb + bytes && pb < pa + bytes;
}

}  // namespace

namespace ommp {

// Resolves the scratch address on the current device.  Called when a system
// is set up on a device, so that a later ommp_gpu_tmatvec_noalloc call on it
// neither loads a module nor places the array.
int noalloc_prepare_device() {
  double *p = nullptr;
  return scratch_address(&p);
}

}  // namespace ommp

extern "C" int32_t ommp_gpu_tmatvec_noalloc(OMMP_SYSTEM_PRT sp, const double *x_dev, double *y_dev, int32_t nrhs,
                                            int32_t dodiag) {
  ommp::System *s = static_cast<ommp::System *>(sp);
  if (!s || !x_dev || !y_dev) {
    ommp::set_last_error("ommp_gpu_tmatvec_noalloc: null system or device pointer");
    return ommp::kErrBadArg;
  }
  if (nrhs < 1 || nrhs > 2) {
    ommp::set_last_error("ommp_gpu_tmatvec_noalloc: nrhs must be 1 or 2");
    return ommp::kErrBadArg;
  }
  const ommp::gpu::DevSites &d = s->dev();
  if (d.n == 0) return ommp::kOk;
  // the finishing kernel reads x at the scaled-pair neighbours of a site
  // while other threads already write y: x and y must be disjoint
  if (ranges_overlap(x_dev, y_dev, (size_t)nrhs * (size_t)d.n * 3 * sizeof(double))) {
    ommp::set_last_error("ommp_gpu_tmatvec_noalloc: x and y overlap (an in-place product is not supported)");
    return ommp::kErrBadArg;
  }
  // the pair kernel needs nsplit * nrhs * n * 3 doubles of partials
  size_t per_split = (size_t)nrhs * (size_t)d.n * 3;
  size_t fit = kNoAllocScratchDoubles / per_split;
  if (fit < 1) {
    ommp::set_last_error("ommp_gpu_tmatvec_noalloc: " + std::to_string(d.n) + " polarizable sites x " +
                         std::to_string(nrhs) + " right-hand sides exceed the 16 MiB static scratch (at most " +
                         std::to_string(kNoAllocScratchDoubles / (3 * (size_t)nrhs)) + " sites)");
    return ommp::kErrBadArg;
  }
  double *scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st) return st;
  if (d.n >= 2048 && ommp::gpu::tmu_sym_scratch_doubles(d, nrhs) <= kNoAllocScratchDoubles) {
    // each unordered pair once, fixed-point sums in the static scratch
    ommp::gpu::launch_tmu_f64_sym(d, nrhs, x_dev, y_dev, dodiag != 0, scratch, s->stream());
  } else {
    int nsplit = ommp::gpu::tmu_pick_split(d, nrhs, ommp::gpu::sm_count(), false);
    if ((size_t)nsplit > fit) nsplit = (int)fit;
    ommp::gpu::launch_tmu_f64(d, nrhs, x_dev, y_dev, dodiag != 0, scratch, nsplit, s->stream());
  }
  cudaError_t e = cudaStreamSynchronize(s->stream());
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("ommp_gpu_tmatvec_noalloc: ") + cudaGetErrorString(e));
    return ommp::kErrCuda;
  }
  return ommp::kOk;
}
