// Flux normalisation and power fields without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while another component owns the
// device memory pool (a coupling framework with its own allocator, a host callback, a
// process that must not grow its device footprint after start-up), or code that issues
// its work into a stream another component records.  pgpu_normalize_power_noalloc gives
// them the normalisation the solvers apply after an eigen-solve (the reference's
// NeutronicSolver::normalizeScalarFlux and calculatePowerAndProductionRate,
// NeutronicSolver.cxx:46-116) on buffers they already own: every input and output is a
// caller-provided device pointer, and the scratch the computation needs lives in a
// file-scope __device__ array of fixed size instead of being allocated.
//
// The scratch holds the raw power of each cell (so the second pass does not recompute it)
// plus the deterministic reduction's block partials and ticket counter.  Its capacity is
// kNoAllocMaxCells cells; larger problems are rejected and must use the allocating path
// (pgpu_problem_solve / pgpu_problem_get_power).  The array exists once per device that
// loads the library and is held until the process exits.
#include <cstring>
#include <mutex>

#include "pgpu_internal.cuh"

namespace pgpu {
namespace {

constexpr int kNoAllocMaxCells = 1 << 20;   // 1,048,576 cells
constexpr int kNoAllocBlocks = 512;         // grid cap: partial sums per reduction

// Layout of the scratch array (in doubles):
//   [0, kNoAllocMaxCells)                raw cell power  sum_g phi kappa_sigma_f V
//   [kNoAllocMaxCells, + 2 * kMaxBlocks) block partial sums of a two-value reduction
//                                        (block_reduce_last strides values by kMaxBlocks)
//   then 8 doubles of scalars: p0, total power, negatives; ticket counter (as bits)
constexpr size_t kPartOff = (size_t)kNoAllocMaxCells;
constexpr size_t kScalOff = kPartOff + 2 * (size_t)kMaxBlocks;
constexpr size_t kScratchDoubles = kScalOff + 8;
static_assert(kNoAllocBlocks <= kMaxBlocks, "grid cap must fit the partial-sum slots");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];  // 8 MiB + 19 KiB

struct NoAllocScratch {
  double* cellp;
  double* partials;
  double* scal;          // scal[0] = p0, scal[1] = total power, scal[2] = negatives
  unsigned int* ticket;  // in scal[4]
};

NoAllocScratch view_of(double* base) {
  NoAllocScratch s;
  s.cellp = base;
  s.partials = base + kPartOff;
  s.scal = base + kScalOff;
  s.ticket = reinterpret_cast<unsigned int*>(base + kScalOff + 4);
  return s;
}

// Pass 1: raw cell power q_raw_i = sum_g phi kappa_sigma_f V into scratch, p0 = sum q_raw.
__global__ void k_na_power(int n, int G, const int* __restrict__ mat, const double* __restrict__ vol,
                           const double* __restrict__ ksf, const double* __restrict__ phi, NoAllocScratch S) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* ks = ksf + (size_t)mat[i] * G;
    double q = 0.0;
    for (int g = 0; g < G; g++) q += phi[(size_t)i * G + g] * ks[g] * vol[i];
    S.cellp[i] = q;
    acc[0] += q;
  }
  ReduceSlots<1> slots{S.partials, S.ticket};
  double tot[1];
  if (block_reduce_last<1>(acc, slots, tot) && threadIdx.x == 0) S.scal[0] = tot[0];
}

// Pass 2: phi_out = phi * power / p0, q = q_raw * power / p0, P = sum_g phi_out nu_sigma_f V / k,
// total power and the count of negative entries.  A flux without a positive, finite power
// (p0 <= 0, NaN or Inf: no fissile material, an all-zero or broken flux) cannot be
// normalised: every output is set to zero and the negatives count to -1, the marker the
// caller checks (the call itself returns before the kernels run).
__global__ void k_na_fields(int n, int G, const int* __restrict__ mat, const double* __restrict__ vol,
                            const double* __restrict__ nsf, const double* __restrict__ phi, double power,
                            double keff, double* phi_out, double* q, double* P, NoAllocScratch S,
                            double* total_out, int* negatives_out) {
  const double p0 = S.scal[0];
  const bool bad = !(p0 > 0.0) || !isfinite(p0);
  const double f = bad ? 0.0 : power / p0;
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* ns = nsf + (size_t)mat[i] * G;
    const double V = vol[i];
    double Pi = 0.0;
    for (int g = 0; g < G; g++) {
      const double v = bad ? 0.0 : phi[(size_t)i * G + g] * f;
      phi_out[(size_t)i * G + g] = v;
      if (v < 0.0) acc[1] += 1.0;
      Pi += v * ns[g] * V / keff;
    }
    const double qi = bad ? 0.0 : S.cellp[i] * f;
    q[i] = qi;
    P[i] = Pi;
    acc[0] += qi;
  }
  ReduceSlots<2> slots{S.partials, S.ticket};
  double tot[2];
  if (block_reduce_last<2>(acc, slots, tot) && threadIdx.x == 0) {
    S.scal[1] = tot[0];
    S.scal[2] = bad ? -1.0 : tot[1];
    if (total_out) *total_out = tot[0];
    if (negatives_out) *negatives_out = bad ? -1 : (int)tot[1];
  }
}

// Device address of the scratch array, looked up once per device with that device current.
std::mutex g_noalloc_mutex;
double* g_noalloc_addr[64] = {nullptr};

int scratch_address(int device, double** out) {
  if (device < 0 || device >= 64) return fail(PGPU_ERR_INVALID, "device index out of range for the no-alloc path");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(PGPU_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
    g_noalloc_addr[device] = static_cast<double*>(ptr);
  }
  *out = g_noalloc_addr[device];
  return PGPU_OK;
}

}  // namespace
}  // namespace pgpu

extern "C" {

int pgpu_normalize_power_noalloc(int num_cells, int num_groups, const int* materials, const double* volumes,
                                 const double* kappa_sigma_f, const double* nu_sigma_f, const double* phi,
                                 double power, double keff, double* phi_out, double* q, double* P,
                                 double* total_power, int* negatives, void* stream) {
  using namespace pgpu;
  if (num_cells < 1 || num_groups < 1) return fail(PGPU_ERR_INVALID, "pgpu_normalize_power_noalloc: bad sizes");
  if (num_cells > kNoAllocMaxCells)
    return fail(PGPU_ERR_INVALID, "pgpu_normalize_power_noalloc: " + std::to_string(num_cells) +
                                      " cells exceed the fixed scratch capacity of " + std::to_string(kNoAllocMaxCells) +
                                      " cells; use the allocating path");
  if (!materials || !volumes || !kappa_sigma_f || !nu_sigma_f || !phi || !phi_out || !q || !P || !(keff > 0.0))
    return fail(PGPU_ERR_INVALID, "pgpu_normalize_power_noalloc: null buffer or non-positive keff");
  // The work runs on the device that owns `stream` (the current device for the legacy
  // default stream); the scratch address is that device's, looked up with it current.
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int current = 0, device = 0;
  PGPU_CUDA(cudaGetDevice(&current));
  device = current;
  if (s) PGPU_CUDA(cudaStreamGetDevice(s, &device));
  if (device != current) PGPU_CUDA(cudaSetDevice(device));
  double* base = nullptr;
  int st = scratch_address(device, &base);
  if (st == PGPU_OK) {
    NoAllocScratch S = view_of(base);
    // the ticket counter must start at zero; the previous call's values are otherwise kept
    cudaError_t e = cudaMemsetAsync(S.ticket, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
      const int blocks = std::min(kNoAllocBlocks, (num_cells + kThreads - 1) / kThreads);
      k_na_power<<<blocks, kThreads, 0, s>>>(num_cells, num_groups, materials, volumes, kappa_sigma_f, phi, S);
      k_na_fields<<<blocks, kThreads, 0, s>>>(num_cells, num_groups, materials, volumes, nu_sigma_f, phi, power,
                                              keff, phi_out, q, P, S, total_power, negatives);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess)
      st = fail(PGPU_ERR_CUDA, std::string("pgpu_normalize_power_noalloc: ") + cudaGetErrorString(e));
  }
  if (device != current) cudaSetDevice(current);
  return st;
}

}  // extern "C"
