// fvx_runtime.cu -- library state behind the C ABI: error strings, the device
// status word, per-device facts, and the host-pointer context (persistent
// device workspace + pinned staging) used by the fvx_host_* entries.
//
// The reference re-uploads every input with one wp.array() per array and
// downloads with a blocking .numpy() on every call
// (src/fluxvortex/warp_kernels.py:196-214).  A host call here packs all
// inputs into one pinned staging block, issues a single host-to-device copy,
// runs the kernels, and issues a single device-to-host copy, on a stream and
// a workspace that persist for the life of the context.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "fvx_common.cuh"

namespace fvx {

namespace {
std::vector<StatusReader>& status_readers() {
  static std::vector<StatusReader> v;
  return v;
}
}  // namespace

void register_status_reader(StatusReader fn) { status_readers().push_back(fn); }

namespace {
std::atomic<unsigned long long> g_launches{0};
}
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {
thread_local char t_err[512] = "";
std::mutex g_dev_mu;
std::vector<int> g_sm_count;
std::vector<int> g_smem_optin;
}  // namespace

void set_last_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
}

int device_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (dev >= static_cast<int>(g_sm_count.size())) g_sm_count.resize(dev + 1, 0);
  if (g_sm_count[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    g_sm_count[dev] = n;
  }
  return g_sm_count[dev];
}

int device_smem_optin() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 48 * 1024;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (dev >= static_cast<int>(g_smem_optin.size())) g_smem_optin.resize(dev + 1, 0);
  if (g_smem_optin[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        n <= 0)
      n = 48 * 1024;
    g_smem_optin[dev] = n;
  }
  return g_smem_optin[dev];
}

int segments_collapsed_launch(const double*, int64_t, const double*, const double*,
                              const double*, const double*, const double*, const double*,
                              const double*, double, int64_t, int, double*, int64_t*, void*,
                              size_t, cudaStream_t);
size_t segments_collapsed_scratch(int64_t, int64_t);
int segments_expanded_launch(const double*, int64_t, const double*, const double*,
                             const double*, const double*, const double*, const double*,
                             const double*, double, int64_t, int, double*, int64_t*,
                             cudaStream_t);
size_t particle_pairs_scratch(int, int, int64_t, int64_t);
int particle_pairs_launch(int, int, int, const double*, const double*, int64_t, const double*,
                          const double*, const double*, int64_t, double*, double*, void*,
                          size_t, cudaStream_t);

}  // namespace fvx

struct fvx_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  void* dbuf = nullptr;
  size_t dcap = 0;
  void* hbuf = nullptr;
  size_t hcap = 0;
  std::mutex mu;
};

namespace {

constexpr size_t kAlign = 256;
size_t round_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// Packs host arrays back to back (256-byte aligned) into the pinned staging
// buffer; the device copy keeps the same offsets.
struct Packer {
  std::vector<std::pair<const void*, size_t>> items;
  size_t total = 0;
  size_t add(const void* p, size_t bytes) {
    size_t off = total;
    items.emplace_back(p, bytes);
    total = round_up(total + bytes);
    return off;
  }
};

int ensure(fvx_context* c, size_t dbytes, size_t hbytes) {
  if (dbytes > c->dcap) {
    if (c->dbuf) cudaFree(c->dbuf);
    c->dbuf = nullptr;
    c->dcap = 0;
    size_t cap = round_up(dbytes + dbytes / 4);
    FVX_CUDA_TRY(cudaMalloc(&c->dbuf, cap));
    c->dcap = cap;
  }
  if (hbytes > c->hcap) {
    if (c->hbuf) cudaFreeHost(c->hbuf);
    c->hbuf = nullptr;
    c->hcap = 0;
    size_t cap = round_up(hbytes + hbytes / 4);
    FVX_CUDA_TRY(cudaMallocHost(&c->hbuf, cap));
    c->hcap = cap;
  }
  return FVX_OK;
}

// Copies the packed inputs to the device workspace (one transfer).
int upload(fvx_context* c, const Packer& pk) {
  char* h = static_cast<char*>(c->hbuf);
  size_t off = 0;
  for (auto& it : pk.items) {
    if (it.first && it.second) std::memcpy(h + off, it.first, it.second);
    off = round_up(off + it.second);
  }
  if (pk.total)
    FVX_CUDA_TRY(cudaMemcpyAsync(c->dbuf, c->hbuf, pk.total, cudaMemcpyHostToDevice, c->stream));
  return FVX_OK;
}

template <typename T>
T* dptr(fvx_context* c, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(c->dbuf) + off);
}

struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DevGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

int host_segments(fvx_context* c, bool expanded, const double* points, int64_t n_points,
                  const double* br, const double* fr, const double* fl, const double* bl,
                  const double* strengths, const double* r_c0s, const double* ages, double nu,
                  int64_t n_vort, int leg_set, double* out, int64_t* counts) {
  FVX_ARG_CHECK(c != nullptr, "null context");
  FVX_ARG_CHECK(n_points >= 0 && n_vort >= 0, "negative size");
  const size_t out_elems =
      static_cast<size_t>(n_points) * 3 * (expanded ? static_cast<size_t>(n_vort) : 1);
  if (n_points == 0 || n_vort == 0) {
    if (out && out_elems) std::memset(out, 0, out_elems * sizeof(double));
    return leg_set >= 0 && leg_set <= 2 ? FVX_OK : FVX_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  DevGuard g(c->device);
  const size_t pb = sizeof(double) * 3 * n_points, vb = sizeof(double) * 3 * n_vort,
               sb = sizeof(double) * n_vort;
  Packer pk;
  size_t o_p = pk.add(points, pb);
  size_t o_c[4] = {pk.add(br, vb), pk.add(fr, vb), pk.add(fl, vb), pk.add(bl, vb)};
  size_t o_s = pk.add(strengths, sb);
  size_t o_r = pk.add(r_c0s, sb);
  size_t o_a = ages ? pk.add(ages, sb) : 0;
  const size_t in_bytes = pk.total;
  const size_t out_bytes = round_up(out_elems * sizeof(double));
  const size_t cnt_bytes = round_up(4 * sizeof(int64_t));
  const size_t scratch = expanded ? 0 : round_up(fvx::segments_collapsed_scratch(n_points, n_vort));
  const size_t o_out = in_bytes, o_cnt = o_out + out_bytes, o_scr = o_cnt + cnt_bytes;
  int rc = ensure(c, o_scr + scratch, in_bytes > out_bytes + cnt_bytes ? in_bytes : out_bytes + cnt_bytes);
  if (rc) return rc;
  if ((rc = upload(c, pk))) return rc;
  FVX_CUDA_TRY(cudaMemsetAsync(dptr<char>(c, o_cnt), 0, cnt_bytes, c->stream));
  const double* dpts = dptr<double>(c, o_p);
  const double* dc[4] = {dptr<double>(c, o_c[0]), dptr<double>(c, o_c[1]),
                         dptr<double>(c, o_c[2]), dptr<double>(c, o_c[3])};
  if (expanded)
    rc = fvx::segments_expanded_launch(dpts, n_points, dc[0], dc[1], dc[2], dc[3],
                                       dptr<double>(c, o_s), dptr<double>(c, o_r),
                                       ages ? dptr<double>(c, o_a) : nullptr, nu, n_vort, leg_set,
                                       dptr<double>(c, o_out), dptr<int64_t>(c, o_cnt), c->stream);
  else
    rc = fvx::segments_collapsed_launch(dpts, n_points, dc[0], dc[1], dc[2], dc[3],
                                        dptr<double>(c, o_s), dptr<double>(c, o_r),
                                        ages ? dptr<double>(c, o_a) : nullptr, nu, n_vort,
                                        leg_set, dptr<double>(c, o_out), dptr<int64_t>(c, o_cnt),
                                        dptr<char>(c, o_scr), scratch, c->stream);
  if (rc) return rc;
  // output and counters are adjacent: one device-to-host transfer
  FVX_CUDA_TRY(cudaMemcpyAsync(c->hbuf, dptr<char>(c, o_out), out_bytes + cnt_bytes,
                               cudaMemcpyDeviceToHost, c->stream));
  FVX_CUDA_TRY(cudaStreamSynchronize(c->stream));
  std::memcpy(out, c->hbuf, out_elems * sizeof(double));
  if (counts) {
    const int64_t* hc = reinterpret_cast<const int64_t*>(static_cast<char*>(c->hbuf) + out_bytes);
    for (int k = 0; k < 4; ++k) counts[k] += hc[k];
  }
  return FVX_OK;
}

}  // namespace

extern "C" {

const char* fvx_version(void) { return "fluxvortex_gb300 0.1.0 (sm_103a)"; }

const char* fvx_last_error(void) { return fvx::t_err; }

unsigned long long fvx_launch_count(void) { return fvx::g_launches.load(); }

int fvx_status_read_and_clear(unsigned* bits, void* stream) {
  FVX_ARG_CHECK(bits != nullptr, "null bits");
  *bits = 0u;
  for (fvx::StatusReader fn : fvx::status_readers())
    FVX_CUDA_TRY(fn(bits, static_cast<cudaStream_t>(stream)));
  return FVX_OK;
}

int fvx_context_create(int device, fvx_context** ctx) {
  FVX_ARG_CHECK(ctx != nullptr, "null ctx");
  *ctx = nullptr;
  fvx_context* c = new fvx_context();
  c->device = device;
  DevGuard g(device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    fvx::set_last_error("cudaStreamCreate: %s", cudaGetErrorString(e));
    delete c;
    return FVX_ERR_CUDA;
  }
  *ctx = c;
  return FVX_OK;
}

void fvx_context_destroy(fvx_context* c) {
  if (!c) return;
  {
    DevGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->dbuf) cudaFree(c->dbuf);
    if (c->hbuf) cudaFreeHost(c->hbuf);
    if (c->stream) cudaStreamDestroy(c->stream);
  }
  delete c;
}

int fvx_host_segments_collapsed(fvx_context* ctx, const double* points, int64_t n_points,
                                const double* br, const double* fr, const double* fl,
                                const double* bl, const double* strengths, const double* r_c0s,
                                const double* ages, double nu, int64_t n_vortices, int leg_set,
                                double* out, int64_t* singularity_counts) {
  return host_segments(ctx, false, points, n_points, br, fr, fl, bl, strengths, r_c0s, ages, nu,
                       n_vortices, leg_set, out, singularity_counts);
}

int fvx_host_segments_expanded(fvx_context* ctx, const double* points, int64_t n_points,
                               const double* br, const double* fr, const double* fl,
                               const double* bl, const double* strengths, const double* r_c0s,
                               const double* ages, double nu, int64_t n_vortices, int leg_set,
                               double* out, int64_t* singularity_counts) {
  return host_segments(ctx, true, points, n_points, br, fr, fl, bl, strengths, r_c0s, ages, nu,
                       n_vortices, leg_set, out, singularity_counts);
}

int fvx_host_particle_pairs(fvx_context* c, int mode, int kernel, int precision,
                            const double* tgt_pos, const double* tgt_gamma, int64_t n_targets,
                            const double* src_pos, const double* src_gamma,
                            const double* src_sigma, int64_t n_sources, double* out_a,
                            double* out_b) {
  FVX_ARG_CHECK(c != nullptr, "null context");
  FVX_ARG_CHECK(n_targets >= 0 && n_sources >= 0, "negative size");
  const int nc = mode == FVX_PAIR_VELOCITY_STRETCH ? 6 : mode == FVX_PAIR_JACOBIAN ? 9 : 3;
  const int na = mode == FVX_PAIR_VELOCITY_STRETCH ? 3 : nc;
  if (n_targets == 0) return FVX_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  DevGuard g(c->device);
  const bool need_tg = mode == FVX_PAIR_STRETCH || mode == FVX_PAIR_VELOCITY_STRETCH;
  Packer pk;
  size_t o_t = pk.add(tgt_pos, sizeof(double) * 3 * n_targets);
  size_t o_tg = need_tg ? pk.add(tgt_gamma, sizeof(double) * 3 * n_targets) : 0;
  size_t o_p = pk.add(src_pos, sizeof(double) * 3 * n_sources);
  size_t o_g = pk.add(src_gamma, sizeof(double) * 3 * n_sources);
  size_t o_s = pk.add(src_sigma, sizeof(double) * n_sources);
  const size_t in_bytes = pk.total;
  const size_t a_bytes = round_up(sizeof(double) * na * n_targets);
  const size_t b_bytes = round_up(sizeof(double) * (nc - na) * n_targets);
  const size_t scratch = round_up(fvx::particle_pairs_scratch(mode, precision, n_targets, n_sources));
  const size_t o_a = in_bytes, o_b = o_a + a_bytes, o_scr = o_b + b_bytes;
  int rc = ensure(c, o_scr + scratch, in_bytes > a_bytes + b_bytes ? in_bytes : a_bytes + b_bytes);
  if (rc) return rc;
  if ((rc = upload(c, pk))) return rc;
  rc = fvx::particle_pairs_launch(mode, kernel, precision, dptr<double>(c, o_t),
                                  need_tg ? dptr<double>(c, o_tg) : nullptr, n_targets,
                                  dptr<double>(c, o_p), dptr<double>(c, o_g), dptr<double>(c, o_s),
                                  n_sources, dptr<double>(c, o_a),
                                  nc > na ? dptr<double>(c, o_b) : nullptr, dptr<char>(c, o_scr),
                                  scratch, c->stream);
  if (rc) return rc;
  FVX_CUDA_TRY(cudaMemcpyAsync(c->hbuf, dptr<char>(c, o_a), a_bytes + b_bytes,
                               cudaMemcpyDeviceToHost, c->stream));
  FVX_CUDA_TRY(cudaStreamSynchronize(c->stream));
  std::memcpy(out_a, c->hbuf, sizeof(double) * na * n_targets);
  if (nc > na) std::memcpy(out_b, static_cast<char*>(c->hbuf) + a_bytes,
                           sizeof(double) * (nc - na) * n_targets);
  return FVX_OK;
}

}  // extern "C"
