// pgpu_* entry points shared by both solver kinds: error state, options, problem
// accessors and destruction.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>

#include "pgpu_internal.cuh"

namespace pgpu {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

// The device's default pool keeps up to this many freed bytes for reuse instead of
// returning them to the driver at the next synchronisation (a served stream allocates and
// frees every request's operator).
constexpr unsigned long long kPoolKeepBytes = 4ull << 30;

static void keep_pool_memory() {
  static std::mutex mu;
  static std::set<int> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(mu);
  if (!done.insert(dev).second) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
  unsigned long long keep = kPoolKeepBytes;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
}

int dev_alloc(DevBuf& b, size_t bytes, long long* counter, cudaStream_t stream) {
  b.release();
  if (bytes == 0) bytes = 16;
  cudaError_t e;
  if (stream) {
    keep_pool_memory();
    e = cudaMallocAsync(&b.ptr, bytes, stream);
    // callers may touch the buffer from the host API (synchronous copies and memsets)
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  } else {
    e = cudaMalloc(&b.ptr, bytes);
  }
  if (e != cudaSuccess) {
    if (b.ptr && stream) cudaFreeAsync(b.ptr, stream);
    b.ptr = nullptr;
    return fail(e == cudaErrorMemoryAllocation ? PGPU_ERR_NO_MEMORY : PGPU_ERR_CUDA,
                std::string("device allocation(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
  }
  b.bytes = bytes;
  b.stream = stream;
  if (counter) *counter += (long long)bytes;
  return PGPU_OK;
}

namespace {
struct PinnedScratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  ~PinnedScratch() {
    if (ptr) cudaFreeHost(ptr);
  }
};
thread_local PinnedScratch t_pinned;
}  // namespace

void* pinned_scratch(size_t bytes) {
  if (t_pinned.bytes < bytes) {
    if (t_pinned.ptr) cudaFreeHost(t_pinned.ptr);
    t_pinned.ptr = nullptr;
    t_pinned.bytes = 0;
    const size_t n = std::max<size_t>(bytes, 4096);
    if (cudaMallocHost(&t_pinned.ptr, n) != cudaSuccess) {
      t_pinned.ptr = nullptr;
      return nullptr;
    }
    t_pinned.bytes = n;
  }
  return t_pinned.ptr;
}

int read_small(void* host, const void* dev, size_t n, cudaStream_t s) {
  void* h = pinned_scratch(n);
  if (!h) return fail(PGPU_ERR_CUDA, "page-locked host scratch");
  PGPU_CUDA(cudaMemcpyAsync(h, dev, n, cudaMemcpyDeviceToHost, s));
  PGPU_CUDA(cudaStreamSynchronize(s));
  std::memcpy(host, h, n);
  return PGPU_OK;
}

int dev_upload(DevBuf& b, const void* host, size_t bytes, long long* counter, cudaStream_t stream) {
  int st = dev_alloc(b, bytes, counter, stream);
  if (st != PGPU_OK) return st;
  // on the problem's stream (the legacy default stream would queue the uploads of
  // problems created on different threads behind each other); creators synchronise the
  // stream before handing the problem back, so the host arrays may be freed then
  if (host && bytes) {
    if (stream) PGPU_CUDA(cudaMemcpyAsync(b.ptr, host, bytes, cudaMemcpyHostToDevice, stream));
    else PGPU_CUDA(cudaMemcpy(b.ptr, host, bytes, cudaMemcpyHostToDevice));
  }
  return PGPU_OK;
}

}  // namespace pgpu

extern "C" {

void pgpu_default_options(pgpu_options* opt) {
  std::memset(opt, 0, sizeof(*opt));
  opt->precision = PGPU_FP64;
  opt->tol_k = 1e-10;
  opt->tol_flux = 1e-9;
  opt->max_outer = 5000;
  opt->max_inner = 2000;
  opt->power = 1.0;
  opt->verbose = 0;
  opt->shift = -1.0;
}

const char* pgpu_last_error(void) { return pgpu::g_last_error.c_str(); }

int pgpu_problem_solve_linear(pgpu_problem* p, double lam, const double* b, double* x, const pgpu_options* opt,
                              pgpu_stats* stats) {
  if (!p) return pgpu::fail(PGPU_ERR_INVALID, "null problem");
  if (p->kind != 1) return pgpu::fail(PGPU_ERR_INVALID, "linear solves are available for diffusion problems");
  if (!b || !x) return pgpu::fail(PGPU_ERR_INVALID, "null right-hand side or solution buffer");
  if (!(lam == lam)) return pgpu::fail(PGPU_ERR_INVALID, "lam is NaN");
  pgpu_options def;
  pgpu_default_options(&def);
  if (!opt) opt = &def;
  pgpu_stats local;
  std::memset(&local, 0, sizeof(local));
  if (!stats) stats = &local;
  std::memset(stats, 0, sizeof(*stats));
  PGPU_CUDA(cudaSetDevice(p->device));
  p->launches = 0;
  p->profile = false;
  int st = pgpu::diffusion_solve_linear(p, lam, b, x, opt, stats);
  cudaStreamSynchronize(p->stream);
  stats->launches = p->launches;
  stats->status = st;
  return st;
}

int pgpu_problem_solve(pgpu_problem* p, const pgpu_options* opt, pgpu_stats* stats) {
  if (!p) return pgpu::fail(PGPU_ERR_INVALID, "null problem");
  pgpu_options def;
  pgpu_default_options(&def);
  if (!opt) opt = &def;
  pgpu_stats local;
  std::memset(&local, 0, sizeof(local));
  if (!stats) stats = &local;
  std::memset(stats, 0, sizeof(*stats));
  PGPU_CUDA(cudaSetDevice(p->device));
  p->launches = 0;
  p->profile = opt->profile != 0;
  p->prof_bytes = 0.0;
  p->prof_launches = 0;
  int st = PGPU_ERR_INVALID;
  if (p->kind == 1) st = pgpu::diffusion_solve(p, opt, stats);
  else if (p->kind == 2) st = pgpu::sn_solve(p, opt, stats);
  cudaStreamSynchronize(p->stream);
  stats->launches = p->launches;
  if (p->profile) {
    stats->kernel_seconds = pgpu::prof_collect(p);
    stats->kernel_launches = p->prof_launches;
    stats->kernel_bytes = p->prof_bytes;
    std::snprintf(stats->kernel_name, sizeof(stats->kernel_name), "%s", p->prof_name);
  }
  p->profile = false;
  stats->status = st;
  p->solved = (st == PGPU_OK);
  if (p->solved) p->keff = stats->keff;
  return st;
}

int pgpu_problem_get_keff(pgpu_problem* p, double* keff) {
  if (!p || !p->solved) return pgpu::fail(PGPU_ERR_INVALID, "problem not solved");
  *keff = p->keff;
  return PGPU_OK;
}

int pgpu_problem_get_scalar_flux(pgpu_problem* p, double* phi) {
  if (!p || !p->solved) return pgpu::fail(PGPU_ERR_INVALID, "problem not solved");
  PGPU_CUDA(cudaSetDevice(p->device));
  return p->kind == 1 ? pgpu::diffusion_get_flux(p, phi) : pgpu::sn_get_flux(p, phi);
}

int pgpu_problem_get_angular_flux(pgpu_problem* p, double* psi) {
  if (!p || !p->solved) return pgpu::fail(PGPU_ERR_INVALID, "problem not solved");
  if (p->kind != 2) return pgpu::fail(PGPU_ERR_INVALID, "angular flux exists only for SN problems");
  PGPU_CUDA(cudaSetDevice(p->device));
  return pgpu::sn_get_angular(p, psi);
}

int pgpu_problem_get_power(pgpu_problem* p, double* q, double* P, double* total) {
  if (!p || !p->solved) return pgpu::fail(PGPU_ERR_INVALID, "problem not solved");
  PGPU_CUDA(cudaSetDevice(p->device));
  return p->kind == 1 ? pgpu::diffusion_get_power(p, q, P, total)
                      : pgpu::sn_get_power(p, q, P, total);
}

long long pgpu_problem_device_bytes(pgpu_problem* p) { return p ? p->bytes : 0; }

int pgpu_problem_set_sm_share(pgpu_problem* p, int sms) {
  if (!p || sms < 0) return pgpu::fail(PGPU_ERR_INVALID, "invalid SM share");
  p->sm_share = sms;
  return PGPU_OK;
}

long long pgpu_problem_upload_bytes(pgpu_problem* p) { return p ? p->uploaded : 0; }

void pgpu_problem_destroy(pgpu_problem* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->kind == 1) pgpu::diffusion_destroy(p);
  if (p->kind == 2) pgpu::sn_destroy(p);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

}  // extern "C"
