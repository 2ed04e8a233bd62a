// Internals shared by the pgpu_* translation units: error state, device buffers,
// deterministic block reductions and the problem handle.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "pampa_gb300.h"

namespace pgpu {

// ---------------------------------------------------------------------------------
// Errors: a thread-local message plus a PGPU_* code.
// ---------------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

#define PGPU_CUDA(call)                                                                 \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return ::pgpu::fail(PGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + \
                                             " (" __FILE__ ":" + std::to_string(__LINE__) + ")"); \
  } while (0)

#define PGPU_CHECK(cond, code, msg)                                                     \
  do {                                                                                  \
    if (cond) return ::pgpu::fail(code, msg);                                           \
  } while (0)

// ---------------------------------------------------------------------------------
// Device buffer (RAII).  Allocations are counted per problem.  A buffer that belongs to a
// problem comes from the device's stream-ordered pool on the problem's stream and goes
// back to it in that stream's order: cudaFree would wait for the whole device, which
// stalls every other solve in flight whenever a served request finishes.
// ---------------------------------------------------------------------------------
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;  // owning problem's stream; null: plain cudaMalloc
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) {
      if (stream) cudaFreeAsync(ptr, stream);
      else cudaFree(ptr);
    }
    ptr = nullptr;
    bytes = 0;
    stream = nullptr;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(ptr); }
};

int dev_alloc(DevBuf& b, size_t bytes, long long* counter, cudaStream_t stream = nullptr);

// Page-locked host scratch of the calling thread (grows on demand, freed when the thread
// exits), for the small device-to-host reads of a solve's control scalars.  A read into
// pageable memory goes through the driver's staging path, which solves running on other
// host threads then wait for; from page-locked memory it is a plain DMA on the stream.
void* pinned_scratch(size_t bytes);

// Reads n bytes of device memory (ordered on stream s) into host memory through the
// thread's page-locked scratch; the stream is synchronised.
int read_small(void* host, const void* dev, size_t n, cudaStream_t s);

// Writes a small value to device memory in stream order, as a kernel argument (no host
// buffer has to outlive the call).
template <typename V>
__global__ void k_put(V* dst, V v) {
  *dst = v;
}
int dev_upload(DevBuf& b, const void* host, size_t bytes, long long* counter, cudaStream_t stream = nullptr);

// ---------------------------------------------------------------------------------
// Launch geometry.  152 SMs on GB300; grids are capped at a multiple of the SM count
// and loop grid-stride, so partial-sum arrays have a fixed, small size.
// ---------------------------------------------------------------------------------
constexpr int kThreads = 256;
constexpr int kMaxGrid = 152 * 8;     // default grid cap of grid-stride kernels
constexpr int kMaxBlocks = 152 * 16;  // largest grid of a reducing kernel (partial-sum slots)
constexpr int kMaxGroups = 16;  // groups per cell handled in registers

inline int grid_for(long long work, int threads = kThreads) {
  long long b = (work + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > kMaxGrid) b = kMaxGrid;
  return (int)b;
}

// Block cap of a problem's grids of `threads`-thread blocks: its SM share times the
// blocks of that size one SM holds at 2048 threads (no cap without a share).
inline int grid_cap(int sm_share, int threads = kThreads) {
  if (sm_share <= 0) return kMaxBlocks;
  const int b = sm_share * (2048 / threads);
  return b < 1 ? 1 : (b > kMaxBlocks ? kMaxBlocks : b);
}

inline int grid_for(long long work, int sm_share, int threads) {
  const int b = grid_for(work, threads), c = grid_cap(sm_share, threads);
  return b < c ? b : c;
}

// ---------------------------------------------------------------------------------
// Deterministic multi-value block reduction.  Each block writes NV partial sums; the
// last block to finish (ticket counter) adds the partials in block order and calls
// `finish` with the totals.  The order of additions depends only on the grid size, so
// results are bitwise reproducible from run to run.
// ---------------------------------------------------------------------------------
template <int NV>
struct ReduceSlots {
  double* partials;       // [NV][kMaxBlocks]
  unsigned int* ticket;   // one counter
};

// Sums the first nv (<= NV, the same in every lane) of v over the warp, into lane 0.
template <int NV>
__device__ inline void warp_sum(double (&v)[NV], int nv = NV) {
#pragma unroll
  for (int k = 0; k < NV; k++)
    if (k < nv)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
}

// Returns true in every thread of the last block, with `tot` filled in thread 0..NV-1's
// view (all threads see the same totals through shared memory).  Only the first nv
// values (the same in every thread) are reduced; the others come back as zero.
template <int NV>
__device__ inline bool block_reduce_last(double (&v)[NV], ReduceSlots<NV> slots, double (&tot)[NV], int nv = NV) {
  __shared__ double sh[NV][32];
  __shared__ bool last;
  warp_sum<NV>(v, nv);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++)
      if (k < nv) sh[k][warp] = v[k];
  __syncthreads();
  if (warp == 0) {
    double w[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) w[k] = lane < nw && k < nv ? sh[k][lane] : 0.0;
    warp_sum<NV>(w, nv);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < NV; k++)
        if (k < nv) slots.partials[k * kMaxBlocks + blockIdx.x] = w[k];
      __threadfence();
      unsigned int t = atomicAdd(slots.ticket, 1u);
      last = (t == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // last block: fixed-order sum of the partials
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) acc[k] = 0.0;
  // partials of the other blocks are read through L2 (ld.global.cg), which also lets the
  // loads of one thread overlap
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; k++)
      if (k < nv) acc[k] += __ldcg(slots.partials + k * kMaxBlocks + b);
  warp_sum<NV>(acc, nv);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++)
      if (k < nv) sh[k][warp] = acc[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      if (k >= nv) continue;
      double s = 0.0;
      for (int w2 = 0; w2 < nw; w2++) s += sh[k][w2];
      sh[k][0] = s;
    }
    *slots.ticket = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; k++) tot[k] = k < nv ? sh[k][0] : 0.0;
  return true;
}

// ---------------------------------------------------------------------------------
// Problem handle.
// ---------------------------------------------------------------------------------
struct DiffusionData;
struct SNData;

}  // namespace pgpu

struct pgpu_problem {
  int kind = 0;  // 1 diffusion, 2 SN
  int device = 0;
  int num_cells = 0, num_groups = 0, num_dirs = 0;
  long long bytes = 0;     // device memory held
  long long uploaded = 0;  // host-to-device bytes copied at creation
  cudaStream_t stream = nullptr;
  // SMs this problem sizes its grids for (0: the whole device).  Solves that share the
  // device (a server's slots) take a share each, so that their kernels run side by side
  // instead of each small kernel filling the device and the streams taking turns.
  int sm_share = 0;
  bool solved = false;
  double keff = 0.0;
  pgpu::DiffusionData* diff = nullptr;
  pgpu::SNData* sn = nullptr;
  // kernel launches issued by this problem (all kernels), and the optional timing of the
  // dominant kernel (transport sweep for SN, SpMV for diffusion) with CUDA events on the
  // problem's stream
  long long launches = 0;
  bool profile = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
  double prof_bytes = 0.0;
  long long prof_launches = 0;
  const char* prof_name = "";
};

namespace pgpu {

// Launch a kernel on `s` and count it against the problem.
template <typename... KArgs, typename... Args>
inline void launch(pgpu_problem* p, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                   Args... args) {
  kernel<<<grid, block, 0, s>>>(args...);
  p->launches++;
}

// Record an event pair around a dominant-kernel region when profiling is on.
inline void prof_begin(pgpu_problem* p, cudaEvent_t* e) {
  *e = nullptr;
  if (!p->profile) return;
  cudaEventCreate(e);
  cudaEventRecord(*e, p->stream);
}

inline void prof_end(pgpu_problem* p, cudaEvent_t e0, long long launches, double bytes) {
  if (!p->profile || !e0) return;
  cudaEvent_t e1;
  cudaEventCreate(&e1);
  cudaEventRecord(e1, p->stream);
  p->prof_events.push_back({e0, e1});
  p->prof_launches += launches;
  p->prof_bytes += bytes;
}

// Sum the recorded regions (stream must be synchronised) and release the events.
inline double prof_collect(pgpu_problem* p) {
  double s = 0.0;
  for (auto& pr : p->prof_events) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pr.first, pr.second);
    s += ms * 1e-3;
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  p->prof_events.clear();
  return s;
}

// Per-kind entry points implemented in pgpu_diffusion.cu / pgpu_sn.cu.
int diffusion_solve(pgpu_problem* p, const pgpu_options* opt, pgpu_stats* stats);
int diffusion_solve_linear(pgpu_problem* p, double lam, const double* b, double* x, const pgpu_options* opt,
                           pgpu_stats* stats);
int diffusion_get_flux(pgpu_problem* p, double* phi);
int diffusion_get_power(pgpu_problem* p, double* q, double* P, double* total);
void diffusion_destroy(pgpu_problem* p);

int sn_solve(pgpu_problem* p, const pgpu_options* opt, pgpu_stats* stats);
int sn_get_flux(pgpu_problem* p, double* phi);
int sn_get_angular(pgpu_problem* p, double* psi);
int sn_get_power(pgpu_problem* p, double* q, double* P, double* total);
void sn_destroy(pgpu_problem* p);

}  // namespace pgpu
