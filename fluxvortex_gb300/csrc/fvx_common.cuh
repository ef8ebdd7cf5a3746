// fvx_common.cuh -- shared device helpers for the fluxvortex_gb300 kernels
// (sm_103a): status reporting, bounded mbarrier waits and 1-D TMA bulk copies
// (cp.async.bulk) that stage source tiles into shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fluxvortex_gb300.h"

namespace fvx {

// Number of SMs and other per-device facts, cached by the host layer.
int device_sm_count();
// Largest dynamic shared memory a block may opt in to (bytes).
int device_smem_optin();

// One list of (target cell, source cell) local-expansion pairs of the
// treecode: targets are leaves (or parents of leaves, size h = 2 x leaf size),
// each pair's expansion added into local[target][32].
struct FarPairs {
  const int* pair_tgt;       // target id of each pair
  const int* pair_cell;      // global source cell id of each pair
  const uint32_t* tgt_key;   // Morton key of each target
  float h;                   // target size
  float* local;              // [targets][32] local expansions (accumulated)
  int n;                     // pairs
};

// Classes of the local-expansion pairs for the FP64 judge: the pair's list
// (0: the leaves' own pairs, 1: the pairs shared through parents of leaves)
// x whether the source cell is larger than the target x four bins of the
// opening ratio mu = sqrt(3)/2 (h_T + h_S) / d against the path's theta
// (every pair on the path has mu < theta): mu/theta in [0.9, 1), [0.8, 0.9),
// [0.65, 0.8) and below 0.65.  The truncation error grows with mu, so the
// classes keep pairs of different error apart.
constexpr int kJudgeClasses = 16;
__host__ __device__ __forceinline__ int judge_class(int list, float hT, float hS, float d2,
                                                    float inv_theta2) {
  const float q = 0.75f * (hT + hS) * (hT + hS) * inv_theta2 / d2;  // (mu / theta)^2
  const int bin = q >= 0.81f ? 0 : (q >= 0.64f ? 1 : (q >= 0.4225f ? 2 : 3));
  return (list << 3) | (hS > hT ? 4 : 0) | bin;
}

// What the FP64 judge decided for each class: the translation and network
// kernels work out each pair's class and read its action from `act`:
// 0 = analytic translation + network residual, 1 = analytic translation
// alone (the network is dropped for the class), 2 = no expansion -- the
// translation kernel queues the pair, (target | list << 30, cell), in `fb`
// for the FP64 direct sum.  act == nullptr: every pair takes action 0.
struct FarJudge {
  const uint8_t* act = nullptr;  // [kJudgeClasses]
  float inv_theta2 = 0.f;        // 1 / theta^2 of the path
  int2* fb = nullptr;
  int* nfb = nullptr;
  int fb_cap = 0;
};

// The judge's stratified sample of local-expansion pairs: per list (0: the
// leaves' own pairs, 1: the pairs shared through parents of leaves) `cap`
// slots, of which the first cnt[list] are used.
struct JudgeSampleView {
  const int* cnt;            // [2] samples per list (device)
  int cap;                   // slots per list
  const int* cell[2];        // source cell of each sample
  const uint32_t* key[2];    // Morton key of its target
  float h[2];                // target size of each list
};

// Thread-local error message of the last failing C-ABI call.
void set_last_error(const char* fmt, ...);

// Counts kernel launches issued by the library (all threads).
void note_launch();

// Device status word: kernels OR bits in here instead of trapping.  The host
// reads and clears it with fvx_status_read_and_clear().  Without relocatable
// device code every translation unit has its own copy (internal linkage);
// each registers a host-side reader at load time.
enum : unsigned {
  kStatusTimeout = 1u,       // a bounded mbarrier wait ran out
  kStatusNonFinite = 2u,     // NaN/Inf met where the reference guards it
  kStatusCapacity = 4u,      // a capacity limit was hit on the device
};
static __device__ unsigned g_status = 0u;

using StatusReader = cudaError_t (*)(unsigned* bits, cudaStream_t stream);
void register_status_reader(StatusReader fn);

namespace {
// ORs this translation unit's status word into *bits and clears it.
cudaError_t read_clear_status_tu(unsigned* bits, cudaStream_t s) {
  unsigned v = 0u, zero = 0u;
  cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_status, sizeof(unsigned), 0,
                                            cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbolAsync(g_status, &zero, sizeof(unsigned), 0, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  *bits |= v;
  return e;
}
struct StatusRegistrar {
  StatusRegistrar() { register_status_reader(&read_clear_status_tu); }
};
StatusRegistrar g_status_registrar;
}  // namespace

// Spin limit of every mbarrier wait (iterations of try_wait, each of which
// already suspends for a hardware-chosen interval).
constexpr uint32_t kWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Returns true once the phase with parity `parity` has completed; false after
// kWaitLimit polls (the caller records kStatusTimeout and skips its work).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint32_t addr = smem_u32(bar);
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 1-D bulk copy global -> shared, completion signalled on `bar` as tx bytes.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void flag_status(unsigned bits) { atomicOr(&g_status, bits); }

// 1/sqrt(x) as the single approximate hardware instruction with subnormal
// inputs and results flushed to zero: for arguments that are normal floats
// (r^2 + sigma^2 with sigma >= 1e-6), the same value as rsqrtf without its
// subnormal handling.
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }

__host__ __device__ __forceinline__ bool aligned16(const void* p) {
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// ---------------------------------------------------------------------------
// Tile stager: copies `count` records of `rec_bytes` bytes each (records
// [first, first+count) of a packed array) into shared memory.  The 16-byte
// aligned prefix goes by one TMA bulk copy issued by thread 0 and tracked on
// `bar`; any ragged tail (at most one record when rec_bytes = 8 or 24) is
// copied by ordinary loads.  Returns the tx bytes the bulk copy will deliver.
//
// Usage per tile and buffer: thread 0 calls mbar_arrive_expect_tx(bar, total)
// after issuing all bulk copies of the tile; every thread later waits on the
// phase, then runs the plain tail copy and a __syncthreads().
struct BulkPlan {
  uint32_t bulk_bytes;  // bytes moved by the bulk copy
  uint32_t tail_bytes;  // bytes left for plain loads
};

__host__ __device__ __forceinline__ BulkPlan plan_bulk(const void* base, int64_t first,
                                                       int count, int rec_bytes, bool use_tma) {
  uint32_t total = static_cast<uint32_t>(count) * static_cast<uint32_t>(rec_bytes);
  const char* src = static_cast<const char*>(base) + first * rec_bytes;
  if (!use_tma || !aligned16(src)) return BulkPlan{0u, total};
  uint32_t bulk = total & ~15u;
  return BulkPlan{bulk, total - bulk};
}

// Plain cooperative copy of `bytes` bytes (8-byte granules) starting at byte
// `offset` of the record run; used for the ragged tail and the no-TMA path.
__device__ __forceinline__ void plain_copy8(void* dst, const void* src, uint32_t offset,
                                            uint32_t bytes) {
  const double* s = reinterpret_cast<const double*>(static_cast<const char*>(src) + offset);
  double* d = reinterpret_cast<double*>(static_cast<char*>(dst) + offset);
  for (uint32_t i = threadIdx.x; i < bytes / 8u; i += blockDim.x) d[i] = s[i];
}

}  // namespace fvx

// Error-checking helpers for the C-ABI layer.
#define FVX_CUDA_TRY(expr)                                                        \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess) {                                                      \
      ::fvx::set_last_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                            __FILE__, __LINE__);                                  \
      return FVX_ERR_CUDA;                                                        \
    }                                                                             \
  } while (0)

// Follows every kernel launch of the library: checks it and counts it (the
// count is what fvx_launch_count() reports).
#define FVX_LAUNCH_CHECK()                                                       \
  do {                                                                           \
    cudaError_t _e = cudaGetLastError();                                         \
    if (_e != cudaSuccess) {                                                     \
      ::fvx::set_last_error("kernel launch failed: %s (%s:%d)",                  \
                            cudaGetErrorString(_e), __FILE__, __LINE__);         \
      return FVX_ERR_CUDA;                                                       \
    }                                                                            \
    ::fvx::note_launch();                                                        \
  } while (0)

#define FVX_ARG_CHECK(cond, ...)                 \
  do {                                           \
    if (!(cond)) {                               \
      ::fvx::set_last_error(__VA_ARGS__);        \
      return FVX_ERR_ARG;                        \
    }                                            \
  } while (0)
