// fvx_noalloc.cu -- the collapsed line-vortex sweep without any allocation.
//
// Who needs this: callers that may not allocate device memory once they are
// running.  Examples are a host program that owns the GPU memory budget and
// hands a plugin nothing but its input and output buffers, and a fixed-rate
// time-stepping loop in which cudaMalloc/cudaFree (which can synchronise the
// whole device) would add unpredictable stalls.  fvx_segments_collapsed needs
// a scratch buffer for its per-split partial sums whenever the target points
// alone cannot fill the GPU, and expects the caller to supply it.  The entry
// point below takes that scratch from a fixed array compiled into this
// library instead, so the caller passes only inputs and outputs and nothing
// here calls cudaMalloc, cudaFree or any other allocating routine.
//
// Limit: the partial sums of one call must fit kScratchBytes (1 MiB); larger
// problems are rejected with FVX_ERR_CAPACITY before anything is launched.
// The array costs 1 MiB of device memory on every GPU that loads the library,
// for the life of the process.
#include <mutex>
#include <vector>

#include "fvx_common.cuh"

namespace fvx {

int segments_collapsed_launch(const double*, int64_t, const double*, const double*,
                              const double*, const double*, const double*, const double*,
                              const double*, double, int64_t, int, double*, int64_t*, void*,
                              size_t, cudaStream_t);
size_t segments_collapsed_scratch(int64_t, int64_t);

namespace {

constexpr size_t kScratchBytes = size_t(1) << 20;

// The shared scratch.  Every call reuses it and it keeps whatever the last
// call left; nothing in it has to start at zero, because each partial sum is
// written by the sweep kernel before the reduction kernel reads it.  Calls that
// overlap on the GPU (different streams, or several host threads) race on it.
static __device__ __align__(256) double g_noalloc_scratch[kScratchBytes / sizeof(double)];

std::mutex g_mu;
std::vector<void*> g_addr;  // device address of g_noalloc_scratch, per device

// On the host the array's name stands for a host-side shadow, not a device
// address.  Resolve the real address once per device, with that device
// current, and cache it.
int scratch_address(void** out) {
  int dev = 0;
  FVX_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev >= static_cast<int>(g_addr.size())) g_addr.resize(dev + 1, nullptr);
  if (g_addr[dev] == nullptr) {
    void* p = nullptr;
    FVX_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return FVX_OK;
}

}  // namespace
}  // namespace fvx

extern "C" int fvx_segments_collapsed_noalloc(const double* points, int64_t n_points,
                                              const double* br, const double* fr,
                                              const double* fl, const double* bl,
                                              const double* strengths, const double* r_c0s,
                                              const double* ages, double nu, int64_t n_vortices,
                                              int leg_set, double* out,
                                              int64_t* singularity_counts, void* stream) {
  // Bad arguments are reported as such, before the size check can mistake
  // them for a capacity problem.
  FVX_ARG_CHECK(leg_set == FVX_LEGS_RING || leg_set == FVX_LEGS_CHORDWISE ||
                    leg_set == FVX_LEGS_HORSESHOE,
                "unknown leg set %d", leg_set);
  FVX_ARG_CHECK(n_points >= 0 && n_vortices >= 0, "negative size");
  const size_t need = fvx::segments_collapsed_scratch(n_points, n_vortices);
  if (need > fvx::kScratchBytes) {
    fvx::set_last_error(
        "fvx_segments_collapsed_noalloc: %lld points x %lld vortices need %zu bytes of "
        "partial sums, more than its fixed %zu-byte scratch; call fvx_segments_collapsed "
        "with a caller-provided scratch buffer instead",
        static_cast<long long>(n_points), static_cast<long long>(n_vortices), need,
        fvx::kScratchBytes);
    return FVX_ERR_CAPACITY;
  }
  void* scratch = nullptr;
  int rc = fvx::scratch_address(&scratch);
  if (rc != FVX_OK) return rc;
  return fvx::segments_collapsed_launch(points, n_points, br, fr, fl, bl, strengths, r_c0s, ages,
                                        nu, n_vortices, leg_set, out, singularity_counts,
                                        scratch, fvx::kScratchBytes,
                                        static_cast<cudaStream_t>(stream));
}
