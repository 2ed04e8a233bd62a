// Discrete-ordinates (SN) k-eigenvalue solve on one GPU.
//
// Replaces the monolithic assembly + LU + Krylov-Schur of SNSolver (SNSolver.cxx:344-670,
// petsc.cxx:175-204) with a matrix-free operator and transport sweeps.  The eigenpair is
// that of the reference's operator R x = (1/k) F x:
//   R[(i,g,m),(i,g,m)]  = sigma_t V + face terms          (SNSolver.cxx:397, 445-597)
//   R[(i,g,m),(i,g2,m2)] -= sigma_s(g2->g) w_m2 V         (isotropic scattering, :417-431)
//   F[(i,g,m),(i,g2,m2)]  = chi_g nu_sigma_f(g2) w_m2 V   (:434-439)
// Face terms per face f with mu = Omega_m . n_f and area A:
//   interior: R[l,l] += w_i mu A, R[l,(j,g,m)] += w_j mu A, (w_i, w_j) = Gauss weights by sign(mu)
//   vacuum:   mu > 0: R[l,l] += mu A, plus the LS boundary correction when enabled
//   reflective: mu > 0: R[l,l] += mu A; else R[l,(i,g,m')] += mu A, m' the reflected direction.
//
// Two solution paths:
//  * scalar-flux space (pure upwind, no LS): with scattering and fission isotropic, the
//    eigenproblem closes on phi0 = sum_m w_m psi plus the incoming angular flux at
//    reflective faces.  One transport sweep inverts the streaming+collision part exactly,
//    so the inner solves are GMRES on (I - T S) over n*G (+ boundary) unknowns, each
//    iteration one sweep.  psi itself is rebuilt by one final sweep.
//  * angular-flux space (general: any Gauss weight delta, LS correction): right-
//    preconditioned GMRES on R psi = b with the matrix-free R and a sweep over the upwind
//    part of R as preconditioner.
// Sweeps follow per-direction upwind level sets built once at setup (Kahn's algorithm
// over the face graph); directions whose faces see the same upwind pattern share one
// schedule, so a Cartesian mesh has 8 (one per octant).  All schedules advance together,
// one kernel launch per level.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "pgpu_internal.cuh"

namespace pgpu {

// ---------------------------------------------------------------------------------
// Device-side operator description
// ---------------------------------------------------------------------------------
template <typename T>
struct SNOp {
  int n, G, M, F;
  int use_ls;
  const int* __restrict__ nf;        // [n]
  const int* __restrict__ kind;      // [F][n]
  const int* __restrict__ nbr;       // [F][n]
  const T* __restrict__ area;        // [F][n]
  const T* __restrict__ nrm;         // [F][n][3]
  const T* __restrict__ gauss;       // [F][n][4]
  const int* __restrict__ raxis;     // [F][n]
  const int* __restrict__ rslot;     // [F][n] reflective-face slot or -1
  const T* __restrict__ lsw;         // [F][n][F] or null
  const T* __restrict__ lsdiag;      // [F][n] sum of LS weights over physical neighbours
  const int* __restrict__ mat;       // [n]
  const T* __restrict__ vol;         // [n]
  const T* __restrict__ dirs;        // [M][3]
  const T* __restrict__ w;           // [M]
  const int* __restrict__ refl;      // [M][3]
  const T* __restrict__ st;          // [nm][G]
  const T* __restrict__ ss;          // [nm][G][G]
  const T* __restrict__ chi;         // [nm][G]
  const T* __restrict__ nsf;         // [nm][G]
  // incoming directions of the reflective slots: a slot's list (one per distinct normal
  // among reflective faces) holds the directions with mu <= 0; the reflective inflow
  // bnd[s][g][k] is stored for those only (k < Mh, zero padded)
  const int* __restrict__ rkind;     // [nrefl] list of slot s
  const int* __restrict__ kmap;      // [nlists][M] position of direction m in a list, -1 if outgoing
  const int* __restrict__ klist;     // [nlists][Mh] directions of a list, -1 padding
  int Mh;
};

// Reflective inflow of slot s, group g, direction m (zero for a direction the slot's list
// does not hold: mu > 0 there, so it is never inflow).
template <typename T>
__device__ __forceinline__ T bnd_val(const SNOp<T>& A, const T* __restrict__ bnd, int s, int g, int m) {
  const int k = A.kmap[A.rkind[s] * A.M + m];
  return k >= 0 ? bnd[((size_t)s * A.G + g) * A.Mh + k] : T(0);
}

struct Schedule {
  int npat = 0, nlev = 0;
  std::vector<int> pat_dirs_ptr, pat_dirs;      // directions of each pattern
  std::vector<int> pat_lev_ptr;                 // per pattern: offset into lev_ptr
  std::vector<int> pat_nlev;
  std::vector<int> lev_ptr;                     // concatenated level offsets (into order)
  std::vector<int> order;                       // concatenated cell orders (n per pattern)
  std::vector<int> grid_x;                      // blocks in x for each global level
};

struct GmresScal {
  double beta;
};

struct SNData {
  int n = 0, G = 0, M = 0, F = 0, nm = 0;
  int use_ls = 0;
  bool upwind = true;       // delta == 1 (no downwind or inflow-side diagonal terms)
  int nrefl = 0;            // reflective face slots
  int Mh = 0;               // incoming directions stored per reflective slot (SNOp)
  DevBuf d_rkind, d_kmap, d_klist;
  Schedule sched;
  // operator (FP64 and FP32 copies of the real-valued arrays)
  DevBuf nf, kind, nbr, raxis, rslot, mat, refl;
  DevBuf area, nrm, gauss, lsw, lsdiag, vol, dirs, w, st, ss, chi, nsf, ksf;
  DevBuf area32, nrm32, gauss32, lsw32, lsdiag32, vol32, dirs32, w32, st32, ss32, chi32, nsf32;
  // sweep face weights (SweepFaces)
  DevBuf cls, mutab, wout, windiag, win, mutab32, wout32, windiag32, win32;
  DevBuf rden, rden32;  // reciprocal sweep diagonals [n*G*M], built on first sweep
  DevBuf sweep_ptrs;    // SweepPtrs block read by the level kernels
  // dataflow tiled sweep of a full Cartesian box (k_sweep_flow), when the operator qualifies
  bool kba = false;
  int kba_nx = 0, kba_ny = 0, kba_ntx = 0, kba_nty = 0, kba_ntz = 0, kba_nd = 0, kba_ntasks = 0, kba_nchunk = 1, kba_gchunk = 1;
  int kba_npat = 0;  // sweep patterns of the dataflow sweep (octants, split into direction chunks)
  int kba_t[3] = {4, 4, 4};                // tile shape (4x4x4 or 8x8x4)
  int ncls = 0;                            // cell classes of the coefficient table (0: per-row rden)
  int flow_grid[2] = {0, 0};               // persistent grid per precision [fp32]
  // column sweep of an extruded mesh (k_sweep_col), when the operator qualifies
  bool col = false;
  int col_nxy = 0, col_nz = 0, col_nd = 0, col_ntasks = 0, col_gchunk = 1, col_nchunk = 1;
  int col_grid[2] = {0, 0};
  DevBuf d_col_up, d_col_zm, d_col_zp, d_col_sz, d_col_order;
  DevBuf d_tiles, d_pat_sign, d_ccls, d_crep, coef, coef32, flow_sync, flow_flags;
  DevBuf d_task_order;  // hand-out order of the dataflow sweep's tasks (null: canonical)
  DevBuf trace_buf;     // timeline of one traced sweep (PGPU_FLOW_TRACE), [ntasks][5]
  int trace_sweep = -1; // which sweep of a solve is traced (-1: none)
  std::string trace_file;
  int flow_sleep = 32;  // back-off between flag polls (ns)
  DevBuf d_fpat_dirs_ptr, d_fpat_dirs;  // directions of the dataflow sweep's patterns
  DevBuf mom;  // per-pattern scalar-flux moments of the dataflow sweep [npat][n*G]
  DevBuf d_tile_cls, d_tile_ncls, d_cell_lcls;  // per-tile class lists (FlowGeom)
  cudaGraphExec_t sweep_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [fp32][iso]
  double* hpin = nullptr;  // pinned host mirror of hbuf (GMRES scalars)
  // GMRES cycles as graphs of conditional Arnoldi steps (see gmres), per precision [fp32]
  cudaGraphExec_t arn_graph[2] = {nullptr, nullptr};
  int arn_step_launches[2] = {0, 0};  // kernels of one captured step
  bool capturing = false;             // sweeps enqueue their kernels into the graph being captured
  DevBuf arn;                         // ArnoldiState
  DevBuf lam_dev;                     // the running solve's Wielandt shift (device scalar)
  void drop_arnoldi_graphs() {
    for (auto& g : arn_graph)
      if (g) cudaGraphExecDestroy(g);
    arn_graph[0] = arn_graph[1] = nullptr;
  }
  ~SNData() {
    for (auto& row : sweep_graph)
      for (auto& g : row)
        if (g) cudaGraphExecDestroy(g);
    drop_arnoldi_graphs();
    if (hpin) cudaFreeHost(hpin);
  }
  bool use_tab = false;
  bool have32 = false;
  // schedule on device
  DevBuf d_pat_dirs_ptr, d_pat_dirs, d_pat_lev_ptr, d_pat_nlev, d_lev_ptr, d_order;
  DevBuf d_slot_cell, d_slot_face;
  // work arrays
  DevBuf psi, psi32;          // angular flux [n*G*M]
  DevBuf phi0, fs, fs_old, phi, q, P, src, src32;  // [n*G] / [n]
  DevBuf partials, ticket, oscal, hbuf;
  // Krylov storage: basis [(m+1)][len], plus work vectors
  DevBuf basis, wvec, xvec, rhs, tmp, scat, phtmp;
  DevBuf x64, r64, rhs64;  // FP64 state, residual and right-hand side of the inner system
  size_t basis_len = 0;
  int restart = 0;
  int krylov_prec = -1;  // element size of the Krylov storage (4 or 8)
  int sweeps = 0;        // sweeps of the running solve
  int reorth = 0;        // Arnoldi steps that needed a second Gram-Schmidt pass
};

struct SNOuter {
  double k, S, change, p0, total_power;
  int negatives, nonfinite;
  unsigned long long amax_phi, amax_psi;  // bit patterns of max |phi0|, max |psi| (>= 0)
};

// Entries of the converged flux whose exact value is zero or tiny (e.g. fast flux in a
// source-free, non-scattering region) come out of an iterative solve as +-(solver
// tolerance).  The reference, which factors R exactly, gets exact (non-negative) values
// there and rejects any negative entry.  Entries within max(kZeroFlush, tol_flux) of the
// maximum are therefore set to zero; anything more negative is a genuine negative flux
// (a mode with sign changes) and is reported.
constexpr double kZeroFlush = 1e-9;

template <typename T>
__global__ void k_absmax(long long N, const T* __restrict__ v, unsigned long long* out) {
  double m = 0.0;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    m = fmax(m, fabs((double)v[l]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// ---------------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T mu_of(const SNOp<T>& A, int f, int i, int m) {
  const T* n = A.nrm + ((size_t)f * A.n + i) * 3;
  const T* d = A.dirs + (size_t)m * 3;
  return d[0] * n[0] + d[1] * n[1] + d[2] * n[2];
}

// One level of the sweep for every pattern (blockIdx.y).  Solves each (cell, g, m) row of
// the upwind part of R: psi = (src - upwind face terms - reflective inflow) / diagonal.
// src is isotropic ([n*G]) when iso != 0, else angular ([n*G*M]).  bnd holds incoming
// angular flux at reflective faces ([nrefl][G][Mh], see SNOp) or is null (treated as zero).
// Per-face sweep weights, precomputed at setup so a face costs one or two FP64 operations
// (GB300's FP64 rate is 1/64 of FP32, and the sweep is FP64-bound):
//   outflow (mu > 0):  den += mu * wout   (interior: Gauss weight c0 * A; vacuum: A, minus the
//                                          LS diagonal share; reflective: A)
//   inflow  (mu <= 0): den += mu * windiag (interior, delta < 1: c2 * A)
//                      num -= mu * win * psi_upwind (interior: c3 * A) or * inflow (reflective: A)
// mu comes from a table over the mesh's distinct face normals when there are at most 255.
template <typename T>
struct SweepFaces {
  const unsigned char* __restrict__ cls;  // [F][n] normal class, or null: mu from the normals
  const T* __restrict__ mutab;            // [ncls][M]
  const T* __restrict__ wout;             // [F][n]
  const T* __restrict__ windiag;          // [F][n]
  const T* __restrict__ win;              // [F][n]
  int upwind;                             // windiag == 0 everywhere
  const T* __restrict__ rden;             // [n*G*M] 1 / diagonal, precomputed (or null)
};

template <typename T>
__device__ __forceinline__ T sweep_mu(const SNOp<T>& A, const SweepFaces<T>& W, int f, int i, int m) {
  return W.cls ? W.mutab[W.cls[(size_t)f * A.n + i] * A.M + m] : mu_of(A, f, i, m);
}

// The sweep's diagonal, sigma_t V + outflow terms + inflow-side diagonal terms, depends on
// the operator only; its reciprocal is stored once per (cell, group, direction) so a sweep
// does no FP64 division and skips the outflow faces.
template <typename T>
__device__ __forceinline__ T sweep_den(const SNOp<T>& A, const SweepFaces<T>& W, int i, int g, int m) {
  T den = A.st[A.mat[i] * A.G + g] * A.vol[i];
  for (int f = 0; f < A.nf[i]; f++) {
    const size_t o = (size_t)f * A.n + i;
    const T mu = sweep_mu(A, W, f, i, m);
    if (mu > T(0)) den += mu * W.wout[o];
    else if (!W.upwind) den += mu * W.windiag[o];
  }
  return den;
}

template <typename T>
__global__ void k_sweep_rden(SNOp<T> A, SweepFaces<T> W, T* rden) {
  const int G = A.G, M = A.M, n = A.n;
  const long long N = (long long)n * G * M;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(l % M);
    const int r = (int)(l / M);
    const int i = r / G, g = r - i * G;
    rden[l] = T(1) / sweep_den(A, W, i, g, m);
  }
}

// Buffers of one sweep, read by every level kernel from device memory so that the level
// launches can be captured once in a CUDA graph and replayed for any buffers.
struct SweepPtrs {
  const void* src;
  const void* bnd;
  void* psi;
  void* mom;  // dataflow sweep: per-pattern scalar-flux moments [npat][n*G], or null
};

__global__ void k_set_sweep_ptrs(SweepPtrs* P, const void* src, const void* bnd, void* psi, void* mom) {
  P->src = src;
  P->bnd = bnd;
  P->psi = psi;
  P->mom = mom;
}

template <typename T>
__global__ void k_sweep_level(SNOp<T> A, SweepFaces<T> W, int level, const int* __restrict__ pat_dirs_ptr,
                              const int* __restrict__ pat_dirs, const int* __restrict__ pat_lev_ptr,
                              const int* __restrict__ pat_nlev, const int* __restrict__ lev_ptr,
                              const int* __restrict__ order, const SweepPtrs* __restrict__ P, int iso) {
  const int p = blockIdx.y;
  if (level >= pat_nlev[p]) return;
  const T* __restrict__ src = static_cast<const T*>(P->src);
  const T* __restrict__ bnd = static_cast<const T*>(P->bnd);
  T* psi = static_cast<T*>(P->psi);
  const int d0 = pat_dirs_ptr[p], nd = pat_dirs_ptr[p + 1] - d0;
  const int* lp = lev_ptr + pat_lev_ptr[p];
  const int c0 = lp[level], nc = lp[level + 1] - c0;
  const int* ord = order + (size_t)p * A.n;
  const int G = A.G, M = A.M, n = A.n;
  const int items = nc * G * nd;  // < 2^31 (checked at setup)
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < items; it += gridDim.x * blockDim.x) {
    const int rest = it / nd;
    const int di = it - rest * nd;
    const int ci = rest / G;
    const int g = rest - ci * G;
    const int i = ord[c0 + ci];
    const int m = pat_dirs[d0 + di];
    const size_t l = ((size_t)i * G + g) * M + m;
    T num = iso ? src[(size_t)i * G + g] : src[l];
    const int nfi = A.nf[i];
    if (W.rden) {
      for (int f = 0; f < nfi; f++) {
        const T mu = sweep_mu(A, W, f, i, m);
        if (mu > T(0)) continue;
        const size_t o = (size_t)f * n + i;
        const int kd = A.kind[o];
        if (kd == PGPU_FACE_INTERIOR) {
          num -= (mu * W.win[o]) * psi[((size_t)A.nbr[o] * G + g) * M + m];
        } else if (kd == PGPU_FACE_REFLECTIVE && bnd) {
          num -= (mu * W.win[o]) * bnd_val(A, bnd, A.rslot[o], g, m);
        }
      }
      psi[l] = num * W.rden[l];
      continue;
    }
    T den = A.st[A.mat[i] * G + g] * A.vol[i];
    for (int f = 0; f < nfi; f++) {
      const size_t o = (size_t)f * n + i;
      const T mu = sweep_mu(A, W, f, i, m);
      if (mu > T(0)) {
        den += mu * W.wout[o];
      } else {
        if (!W.upwind) den += mu * W.windiag[o];
        const int kd = A.kind[o];
        if (kd == PGPU_FACE_INTERIOR) {
          num -= (mu * W.win[o]) * psi[((size_t)A.nbr[o] * G + g) * M + m];
        } else if (kd == PGPU_FACE_REFLECTIVE && bnd) {
          num -= (mu * W.win[o]) * bnd_val(A, bnd, A.rslot[o], g, m);
        }
      }
    }
    psi[l] = num / den;
  }
}

// ---------------------------------------------------------------------------------
// Dataflow tiled sweep for a full Cartesian box (one persistent launch per sweep).
//
// The box is cut into tiles (4x4x4 or 8x8x4 cells).  A task is one tile, one octant and one
// chunk of energy groups (all the pattern's directions for those groups; groups never
// couple inside a sweep).  Tasks are numbered tile diagonal by tile diagonal of the
// octant-oriented tile index (tx' + ty' + tz' = D), so the upwind tasks of a task --
// (tx'-1, ty', tz'), (tx', ty'-1, tz'), (tx', ty', tz'-1), same pattern and chunk --
// always come earlier.  Each CTA takes the next task from an atomic counter, stages the
// tile's source and cell classes in shared memory, waits until the flags of its upwind
// tasks hold this sweep's epoch, loads the inflow on the tile's three upwind faces,
// sweeps the tile through its TX+TY+TZ-2 cell diagonals with the tile's angular flux
// in shared memory, writes psi, publishes its own flag and writes its pattern's share of
// the scalar-flux moment.  A task is taken only by a running CTA, and only after every
// earlier task was taken by a running CTA, so every wait ends; the waits are bounded all
// the same (kFlowSpinLimit): a wait that runs out sets the error word, every later wait
// then returns at once, and the host reports PGPU_ERR_TIMEOUT.
//
// Arithmetic per (cell, group, direction): psi = rd * src + sum over the three inflow
// faces of a_f * psi_upwind, with rd = 1 / diagonal and a_f = -(mu_f * w_in,f) * rd.
// (rd, a_x, a_y, a_z) depend on the cell only through its material, volume and face
// weights, so cells are grouped into classes with equal values and the coefficients are
// read from a small per-class table; a mesh with too many classes uses the per-row
// reciprocal diagonal instead (psi = (src - sum mu_f w_in,f psi_upwind) * rden).
// ---------------------------------------------------------------------------------
constexpr int kFlowSlots = 10;  // (group, direction) slots of one task at most
constexpr int kFlowMaxDirs = 16;  // directions of one task at most (an S8 octant holds 10)
constexpr int kColUp = 4;         // column sweep: lateral inflow faces of a column per pattern, at most
// column sweep: layers per batch (loads, then updates, then the progress flag)
template <typename T>
constexpr int kColBatch() {
  return sizeof(T) == 8 ? 2 : 4;  // measured: 4 / 2 (FP32 / FP64) at 80 registers beat 8 / 4 at 128 and 2 / 2 at 64
}
constexpr int kTileClasses = 16;  // cell classes of a tile whose coefficients are staged
constexpr unsigned int kFlowSpinLimit = 1u << 23;  // ~0.3-0.5 s of polling
constexpr unsigned int kFlowStallLimit = 1u << 12;  // polls of the failure-injection wait (~1 ms)

// Tile shapes: 4x4x4 cells (128 threads) for small boxes, 8x8x4 (256 threads) for large
// ones, where fewer tile hops per sweep pay for the longer in-tile diagonals.  Local
// cell c = lx + TX*(ly + TY*lz); the tables list the cells diagonal by diagonal
// (lx + ly + lz), with the offset of each diagonal.
__constant__ unsigned char c_cell444[64];
__constant__ int c_dptr444[11];
__constant__ unsigned char c_cell884[256];
__constant__ int c_dptr884[19];

template <int TX, int TY, int TZ>
struct TileShape;
template <>
struct TileShape<4, 4, 4> {
  static constexpr int kThreads = 128;
  __device__ static __forceinline__ int cell(int k) { return c_cell444[k]; }
  __device__ static __forceinline__ int dptr(int d) { return c_dptr444[d]; }
};
template <>
struct TileShape<8, 8, 4> {
  static constexpr int kThreads = 256;
  __device__ static __forceinline__ int cell(int k) { return c_cell884[k]; }
  __device__ static __forceinline__ int dptr(int d) { return c_dptr884[d]; }
};

struct FlowSync {
  unsigned int next;   // task counter of the running sweep
  unsigned int epoch;  // sweep number; a task's flag holds it once the task is done
  unsigned int error;  // set when a wait ran out
  // Failure injection for the tests of the bounded wait (0: off).  When it holds t + 1,
  // task t also waits, with the short bound kFlowStallLimit, for this word to become 0,
  // which nothing does during a sweep: that wait runs out, sets the error word, and the
  // solve must report PGPU_ERR_TIMEOUT with the context still usable.  Set per solve from
  // PGPU_DEBUG_SWEEP_STALL.
  unsigned int stall;
  unsigned int trace_on;  // record FlowGeom::trace during this sweep
};

struct FlowGeom {
  int nx, ny, ntx, nty, ntz, npat, nd, ntasks;
  int gchunk, nchunk;                    // groups per task, group chunks per (tile, pattern)
  const int* __restrict__ tiles;         // [ntiles][3] oriented tile coordinates, by diagonal
  const int* __restrict__ pat_sign;      // [npat][3]: +1 sweeps towards +axis, -1 towards -axis
  const int* __restrict__ pat_dirs_ptr;  // [npat + 1]
  const int* __restrict__ pat_dirs;
  const unsigned short* __restrict__ ccls;  // [n] cell class, or null (per-row rden)
  const void* coef;                         // [ncls][G][M][4] (rd, a_x, a_y, a_z) in T
  const int* __restrict__ tile_cls;         // [ntiles][kTileClasses] classes of a tile (absolute index)
  const int* __restrict__ tile_ncls;        // [ntiles] their count, > kTileClasses: not staged
  const unsigned char* __restrict__ cell_lcls;  // [n] a cell's index in its tile's class list
  FlowSync* sync;
  unsigned int* flags;  // [npat][nchunk][ntz][nty][ntx] by oriented tile coordinates
  // order in which tasks are handed out: entry t holds (tile * npat + pattern) * nchunk +
  // chunk; every pattern's tasks appear tile diagonal by tile diagonal (null: that order)
  const int* __restrict__ order;
  int sleep_ns;  // back-off between polls of an upwind flag
  // timeline of one sweep for measurement (PGPU_FLOW_TRACE), or null: per handed-out task
  // the global timer when it was taken, when its upwind wait ended, when its diagonals
  // ended and when it finished, and the SM it ran on
  unsigned long long* trace;
};

__device__ __forceinline__ unsigned long long flow_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int flow_smid() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned int ld_relaxed_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until *flag == epoch (relaxed polling, then one acquire load of the flag);
// returns without waiting once any wait of the sweep ran out.
__device__ __forceinline__ void flow_wait(const unsigned int* flag, unsigned int epoch, unsigned int* error,
                                          unsigned int limit = kFlowSpinLimit, int sleep_ns = 32) {
  for (unsigned int it = 0;; it++) {
    if (ld_relaxed_gpu(flag) == epoch) break;
    if (*(volatile unsigned int*)error) return;
    if (it >= limit) {
      atomicExch(error, 1u);
      return;
    }
    if (sleep_ns > 0) __nanosleep(sleep_ns);
  }
  (void)ld_acquire_gpu(flag);
}

__global__ void k_flow_begin(FlowSync* s) {
  s->next = 0u;
  s->epoch = s->epoch + 1u;
}

__device__ __forceinline__ void flow_load4(const double* __restrict__ p, double (&o)[4]) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}

__device__ __forceinline__ void flow_load4(const float* __restrict__ p, float (&o)[4]) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p));
  o[0] = a.x;
  o[1] = a.y;
  o[2] = a.z;
  o[3] = a.w;
}

// Global coordinates of the tile cell with oriented local coordinates (lx, ly, lz).
template <int TX, int TY, int TZ>
struct FlowTile {
  int bx, by, bz, sx, sy, sz;
  __device__ __forceinline__ int x(int lx) const { return bx + (sx > 0 ? lx : TX - 1 - lx); }
  __device__ __forceinline__ int y(int ly) const { return by + (sy > 0 ? ly : TY - 1 - ly); }
  __device__ __forceinline__ int z(int lz) const { return bz + (sz > 0 ? lz : TZ - 1 - lz); }
};

// Shared memory of one task with S slots and Gc groups: the coefficients of the tile's
// classes, the tile's angular flux with a one-cell halo on its three upwind sides (the
// halo holds the inflow, so every update reads its upwind values at fixed offsets), the
// isotropic source, and per cell its class and global index.
template <typename T>
__host__ __device__ constexpr size_t flow_smem_bytes(int TX, int TY, int TZ, int S, int Gc) {
  return ((size_t)kTileClasses * S * 4 + (size_t)(TX + 1) * (TY + 1) * (TZ + 1) * S + (size_t)TX * TY * TZ * Gc) *
             sizeof(T) +
         (size_t)TX * TY * TZ * 2 * sizeof(int);
}

__device__ __forceinline__ void smem_load4(const float* p, float (&o)[4]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  o[0] = a.x, o[1] = a.y, o[2] = a.z, o[3] = a.w;
}

__device__ __forceinline__ void smem_load4(const double* p, double (&o)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  o[0] = a.x, o[1] = a.y, o[2] = b.x, o[3] = b.y;
}

template <typename T, bool kClass, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TileShape<TX, TY, TZ>::kThreads, 1024 / TileShape<TX, TY, TZ>::kThreads)
    k_sweep_flow(SNOp<T> A, SweepFaces<T> W, FlowGeom K, const SweepPtrs* __restrict__ P, int iso) {
  using Shape = TileShape<TX, TY, TZ>;
  constexpr int kCells = TX * TY * TZ, kDiags = TX + TY + TZ - 2;
  constexpr int kFx = TY * TZ, kFy = TX * TZ, kFz = TX * TY, kFaces = kFx + kFy + kFz;  // upwind face cells
  constexpr int PX = TX + 1, PXY = (TX + 1) * (TY + 1), kPad = PXY * (TZ + 1);
  extern __shared__ __align__(16) unsigned char flow_smem[];
  const int G = A.G, M = A.M, n = A.n, Gc = K.gchunk, nd = K.nd, S = nd * Gc;
  T* tcoef = reinterpret_cast<T*>(flow_smem);              // [kTileClasses][S][4]
  T* tp = tcoef + kTileClasses * S * 4;                    // [kPad][S] padded tile
  T* tsrc = tp + kPad * S;                                 // [kCells][Gc]
  int* tcls = reinterpret_cast<int*>(tsrc + kCells * Gc);  // [kCells] class (local or global)
  int* tgi = tcls + kCells;                                // [kCells] global cell index
  __shared__ int s_task;
  // Tables of the tile shape.  Local cell c = lx + TX (ly + TY lz) sits at padded index
  // (lx+1) + PX (ly+1) + PXY (lz+1); its upwind neighbours are 1, PX and PXY below.
  __shared__ int s_plan[kCells];  // cells diagonal by diagonal: c | padded index << 8
  __shared__ int s_face[kFaces];  // upwind face slots: adjacent cell | halo index << 8 | axis << 24
  __shared__ int s_dptr[kDiags + 1];
  __shared__ T s_w[kFlowMaxDirs];  // quadrature weights of the task's directions
  for (int k = threadIdx.x; k < kCells; k += blockDim.x) {
    const int c = Shape::cell(k);
    s_plan[k] = c | ((c % TX + 1) + PX * ((c / TX) % TY + 1) + PXY * (c / (TX * TY) + 1)) << 8;
  }
  for (int fs = threadIdx.x; fs < kFaces; fs += blockDim.x) {
    int a, c, h;
    if (fs < kFx) {  // x face (ly, lz)
      const int ly = fs % TY, lz = fs / TY;
      a = 0, c = TX * (ly + TY * lz), h = PX * (ly + 1) + PXY * (lz + 1);
    } else if (fs < kFx + kFy) {  // y face (lx, lz)
      const int lx = (fs - kFx) % TX, lz = (fs - kFx) / TX;
      a = 1, c = lx + TX * TY * lz, h = (lx + 1) + PXY * (lz + 1);
    } else {  // z face (lx, ly)
      const int lx = (fs - kFx - kFy) % TX, ly = (fs - kFx - kFy) / TX;
      a = 2, c = lx + TX * ly, h = (lx + 1) + PX * (ly + 1);
    }
    s_face[fs] = c | h << 8 | a << 24;
  }
  for (int k = threadIdx.x; k <= kDiags; k += blockDim.x) s_dptr[k] = Shape::dptr(k);
  const T* __restrict__ src = static_cast<const T*>(P->src);
  const T* __restrict__ bnd = static_cast<const T*>(P->bnd);
  T* psi = static_cast<T*>(P->psi);
  T* mom = static_cast<T*>(P->mom);
  const T* __restrict__ coef = static_cast<const T*>(K.coef);
  const unsigned int epoch = *(volatile unsigned int*)&K.sync->epoch;
  const int nx = K.nx, nxy = K.nx * K.ny, ntiles = K.ntx * K.nty * K.ntz;
  // a sweep that forms moments (scalar-flux space) keeps psi only where it is read again:
  // the tile's downwind faces, which hold the inflow of the downwind tiles and, on the box
  // boundary, the outgoing flux of reflective faces
  const bool all_psi = mom == nullptr;
  // fixed thread -> (slot, cell lane) map; slot = local group * nd + direction index
  const int slot = threadIdx.x % S, cl = threadIdx.x / S, ncl = blockDim.x / S;
  const int gl = slot / nd, di = slot - gl * nd;
  for (;;) {
    if (threadIdx.x == 0) s_task = (int)atomicAdd(&K.sync->next, 1u);
    __syncthreads();
    const int t = s_task;
    if (t >= K.ntasks) return;  // uniform over the CTA
    const bool tr = K.trace && threadIdx.x == 0 && *(volatile unsigned int*)&K.sync->trace_on;
    if (tr) K.trace[(size_t)t * 5] = flow_clock();
    const int tc = K.order ? K.order[t] : t;
    const int jp = tc / K.nchunk, ch = tc - jp * K.nchunk;
    const int j = jp / K.npat, p = jp - j * K.npat;
    const int g0 = ch * Gc, gn = min(Gc, G - g0);
    const int tx = K.tiles[3 * j], ty = K.tiles[3 * j + 1], tz = K.tiles[3 * j + 2];
    const int sx = K.pat_sign[3 * p], sy = K.pat_sign[3 * p + 1], sz = K.pat_sign[3 * p + 2];
    const int atx = sx > 0 ? tx : K.ntx - 1 - tx, aty = sy > 0 ? ty : K.nty - 1 - ty, atz = sz > 0 ? tz : K.ntz - 1 - tz;
    const FlowTile<TX, TY, TZ> tile{atx * TX, aty * TY, atz * TZ, sx, sy, sz};
    const int d0 = K.pat_dirs_ptr[p], ndp = K.pat_dirs_ptr[p + 1] - d0;
    const bool active = cl < ncl && gl < gn && di < ndp;
    const int g = g0 + gl;
    const int m = active ? K.pat_dirs[d0 + di] : 0;
    unsigned int* pflags = K.flags + ((size_t)p * K.nchunk + ch) * ntiles;
    const int tb = (atz * K.nty + aty) * K.ntx + atx;
    const int nk = kClass ? K.tile_ncls[tb] : 0;
    const bool staged = kClass && nk <= kTileClasses;
    // 1. data that does not depend on the upwind tiles, loaded while they finish: the
    //    weights, the cells' global indices, source and classes, the coefficients of the
    //    tile's classes, and the inflow on upwind faces that lie on the box boundary
    if (mom && threadIdx.x < ndp) s_w[threadIdx.x] = A.w[K.pat_dirs[d0 + threadIdx.x]];
    for (int c = threadIdx.x; c < kCells; c += blockDim.x) {
      const int i = tile.x(c % TX) + nx * tile.y((c / TX) % TY) + nxy * tile.z(c / (TX * TY));
      tgi[c] = i;
      if (iso)
        for (int gg = 0; gg < gn; gg++) tsrc[c * Gc + gg] = src[(size_t)i * G + g0 + gg];
      if (kClass) tcls[c] = staged ? (int)K.cell_lcls[i] : (int)K.ccls[i];
    }
    if (staged && active)
      for (int k = cl; k < nk; k += ncl)
        flow_load4(coef + (((size_t)K.tile_cls[(size_t)tb * kTileClasses + k] * G + g) * M + m) * 4,
                   *reinterpret_cast<T(*)[4]>(tcoef + (k * S + slot) * 4));
    const int inner = (tx > 0) | (ty > 0) << 1 | (tz > 0) << 2;  // upwind faces inside the box
    if (active && inner != 7)
      for (int fs = cl; fs < kFaces; fs += ncl) {
        const int e = s_face[fs], a = e >> 24, c = e & 255;
        if ((inner >> a) & 1) continue;
        T val = T(0);
        if (bnd) {
          const int f = a == 0 ? (sx > 0 ? 3 : 1) : (a == 1 ? (sy > 0 ? 0 : 2) : (sz > 0 ? 4 : 5));
          const size_t o = (size_t)f * n + (tile.x(c % TX) + nx * tile.y((c / TX) % TY) + nxy * tile.z(c / (TX * TY)));
          if (A.kind[o] == PGPU_FACE_REFLECTIVE) val = bnd_val(A, bnd, A.rslot[o], g, m);
        }
        tp[((e >> 8) & 0xffff) * S + slot] = val;
      }
    // 2. wait for the upwind tiles of this pattern and chunk
    if (threadIdx.x < 3) {
      const int a = threadIdx.x;
      const int ux = tx - (a == 0), uy = ty - (a == 1), uz = tz - (a == 2);
      if (ux >= 0 && uy >= 0 && uz >= 0)
        flow_wait(pflags + (uz * K.nty + uy) * K.ntx + ux, epoch, &K.sync->error, kFlowSpinLimit, K.sleep_ns);
      if (a == 0 && *(volatile unsigned int*)&K.sync->stall == (unsigned int)t + 1u)
        flow_wait(&K.sync->stall, 0u, &K.sync->error, kFlowStallLimit);  // injected failure: runs out
    }
    __syncthreads();
    if (tr) K.trace[(size_t)t * 5 + 1] = flow_clock();
    // 3. inflow from the upwind tiles (through L2), four loads in flight per thread
    if (active && inner) {
      for (int f0 = cl; f0 < kFaces; f0 += 4 * ncl) {
        T v[4];
        int h[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int fs = f0 + u * ncl;
          v[u] = T(0);
          h[u] = -1;
          if (fs < kFaces) {
            const int e = s_face[fs], a = e >> 24;
            if ((inner >> a) & 1) {
              const int nb = tgi[e & 255] - (a == 0 ? sx : (a == 1 ? sy * nx : sz * nxy));
              v[u] = __ldcg(psi + ((size_t)nb * G + g) * M + m);
              h[u] = (e >> 8) & 0xffff;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (h[u] >= 0) tp[h[u] * S + slot] = v[u];
      }
    }
    __syncthreads();
    // 4. the tile's cell diagonals
    const int fx = sx > 0 ? 3 : 1, fy = sy > 0 ? 0 : 2, fz = sz > 0 ? 4 : 5;
    T mux = T(0), muy = T(0), muz = T(0);
    if (!kClass && active) {
      mux = fabs(A.dirs[(size_t)m * 3]);
      muy = fabs(A.dirs[(size_t)m * 3 + 1]);
      muz = fabs(A.dirs[(size_t)m * 3 + 2]);
    }
    for (int dd = 0; dd < kDiags; dd++) {
      const int cb = s_dptr[dd], cn = s_dptr[dd + 1] - cb;
      if (active)
        for (int q = cl; q < cn; q += ncl) {
          const int e = s_plan[cb + q], c = e & 255;
          const int b = (e >> 8) * S + slot;
          const T ux = tp[b - S], uy = tp[b - PX * S], uz = tp[b - PXY * S];
          T v;
          if (kClass) {
            T cf[4];
            if (staged)
              smem_load4(tcoef + (tcls[c] * S + slot) * 4, cf);
            else
              flow_load4(coef + (((size_t)tcls[c] * G + g) * M + m) * 4, cf);
            v = cf[0] * (iso ? tsrc[c * Gc + gl] : src[((size_t)tgi[c] * G + g) * M + m]);
            v += cf[3] * uz;
            v += cf[2] * uy;
            v += cf[1] * ux;
          } else {
            const int i = tgi[c];
            const size_t l = ((size_t)i * G + g) * M + m;
            T num = iso ? tsrc[c * Gc + gl] : src[l];
            num += (muz * W.win[(size_t)fz * n + i]) * uz;
            num += (muy * W.win[(size_t)fy * n + i]) * uy;
            num += (mux * W.win[(size_t)fx * n + i]) * ux;
            v = num * W.rden[l];
          }
          tp[b] = v;
          if (all_psi || c % TX == TX - 1 || (c / TX) % TY == TY - 1 || c / (TX * TY) == TZ - 1)
            psi[((size_t)tgi[c] * G + g) * M + m] = v;
        }
      __syncthreads();
    }
    // 5. publish the tile, then its scalar-flux moment over this pattern's directions: the
    //    barrier that ended the last diagonal orders every thread's psi stores before thread
    //    0's release store (release is cumulative), which the consumer pairs with an acquire
    if (tr) K.trace[(size_t)t * 5 + 2] = flow_clock();
    if (threadIdx.x == 0) st_release_gpu(pflags + (tz * K.nty + ty) * K.ntx + tx, epoch);
    if (mom) {
      for (int r = threadIdx.x; r < kCells * gn; r += blockDim.x) {
        const int c = r / gn, gg = r - c * gn;
        const T* row = tp + ((c % TX + 1) + PX * ((c / TX) % TY + 1) + PXY * (c / (TX * TY) + 1)) * S + gg * nd;
        T acc = T(0);
        for (int dj = 0; dj < ndp; dj++) acc += s_w[dj] * row[dj];
        mom[(size_t)p * n * G + (size_t)tgi[c] * G + g0 + gg] = acc;
      }
    }
    if (tr) {
      K.trace[(size_t)t * 5 + 3] = flow_clock();
      K.trace[(size_t)t * 5 + 4] = flow_smid();
    }
  }
}

// ---------------------------------------------------------------------------------
// Column sweep of an extruded mesh (see col_plan): one warp per task = (column, sweep
// pattern, chunk of groups); lane = (group of the chunk, direction of the pattern).  The
// task takes the next index from the sweep's atomic counter and walks its layers in the
// pattern's z order, B at a time.  Tasks are pipelined layer batch by layer batch: a
// column publishes how many of its layers are done (with the sweep's epoch in the high
// word), and a column waits (bounded, as the dataflow sweep of Cartesian boxes) only until
// its lateral upwind columns have done the layers of its next batch.  Per batch: the
// loads (cell classes, source, lateral inflow from the upwind columns or the reflective
// inflow, then the coefficient rows), then per layer the update psi = rd q + sum of a_f
// psi_in over the lateral inflow faces in face order, then the z inflow (the layer before
// in sweep order, or the boundary) -- the terms and the order of k_sweep_level_cls.  The
// pattern's share of the scalar-flux moment is summed per (cell, group) in direction
// order.
// ---------------------------------------------------------------------------------
struct ColGeom {
  int nxy, nz, npat, nd, ntasks, gchunk, nchunk;
  const int* __restrict__ up;      // [npat][nxy][kColUp]
  const int* __restrict__ zm;      // [nxy]
  const int* __restrict__ zp;      // [nxy]
  const int* __restrict__ pat_sz;  // [npat]
  const int* __restrict__ pat_dirs_ptr;
  const int* __restrict__ pat_dirs;
  const int* __restrict__ order;   // [ntasks]
  const unsigned short* __restrict__ ccls;
  FlowSync* sync;
  unsigned long long* prog;        // [npat][nchunk][nxy]: epoch << 32 | layers done
  int sleep_ns;
};

__device__ __forceinline__ unsigned long long ld_relaxed_gpu64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_gpu64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Waits until *p >= target (relaxed polling, then one acquire load), as flow_wait.
__device__ __forceinline__ void flow_wait_ge(const unsigned long long* p, unsigned long long target,
                                             unsigned int* error, unsigned int limit, int sleep_ns) {
  for (unsigned int it = 0;; it++) {
    if (ld_relaxed_gpu64(p) >= target) break;
    if (*(volatile unsigned int*)error) return;
    if (it >= limit) {
      atomicExch(error, 1u);
      return;
    }
    if (sleep_ns > 0) __nanosleep(sleep_ns);
  }
  (void)ld_acquire_gpu64(p);
}

template <typename T, int B>
__global__ void __launch_bounds__(128, 6) k_sweep_col(SNOp<T> A, ColGeom K, const T* __restrict__ coef,
                                                   const SweepPtrs* __restrict__ P, int iso) {
  __shared__ T s_mom[4][B][32];  // per warp: w_m psi of the batch's layers, by lane
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const T* __restrict__ src = static_cast<const T*>(P->src);
  const T* __restrict__ bnd = static_cast<const T*>(P->bnd);
  T* psi = static_cast<T*>(P->psi);
  T* mom = static_cast<T*>(P->mom);
  const unsigned long long ep = (unsigned long long)*(volatile unsigned int*)&K.sync->epoch << 32;
  const int G = A.G, M = A.M, n = A.n, F = A.F, nxy = K.nxy, nz = K.nz;
  const int gl = lane / K.nd, di = lane - gl * K.nd;
  for (;;) {
    int t = 0;
    if (lane == 0) t = (int)atomicAdd(&K.sync->next, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= K.ntasks) return;
    const int tc = K.order[t];
    const int cp = tc / K.nchunk, ch = tc - cp * K.nchunk;
    const int c = cp / K.npat, p = cp - c * K.npat;
    const int d0 = K.pat_dirs_ptr[p], ndp = K.pat_dirs_ptr[p + 1] - d0;
    const int g0 = ch * K.gchunk, gn = min(K.gchunk, G - g0);
    const bool active = gl < gn && di < ndp;
    const int g = g0 + gl;
    const int m = active ? K.pat_dirs[d0 + di] : 0;
    const T wm = active ? A.w[m] : T(0);
    int fu[kColUp], cu[kColUp];  // lateral inflow faces and their layer-0 neighbour (-1: boundary)
#pragma unroll
    for (int u = 0; u < kColUp; u++) {
      fu[u] = K.up[((size_t)p * nxy + c) * kColUp + u];
      cu[u] = fu[u] >= 0 ? A.nbr[(size_t)fu[u] * n + c] : -1;
    }
    const int sz = K.pat_sz[p];
    const int fz = sz > 0 ? K.zm[c] : (sz < 0 ? K.zp[c] : -1);  // the z inflow face
    unsigned long long* prog = K.prog + ((size_t)p * K.nchunk + ch) * nxy;
    const bool stall = lane == 0 && *(volatile unsigned int*)&K.sync->stall == (unsigned int)t + 1u;
    T prev = T(0);
    for (int kb = 0; kb < nz; kb += B) {
      const int kn = min(B, nz - kb);
      // wait until the lateral upwind columns have done this batch's layers
      if (lane < kColUp) {
        int c2 = -1;
#pragma unroll
        for (int u = 0; u < kColUp; u++)
          if (u == lane) c2 = cu[u];
        if (c2 >= 0) flow_wait_ge(prog + c2, ep | (unsigned long long)(kb + kn), &K.sync->error, kFlowSpinLimit, K.sleep_ns);
        if (stall && kb == 0) flow_wait(&K.sync->stall, 0u, &K.sync->error, kFlowStallLimit);  // injected failure
      }
      __syncwarp();
      T in[B][kColUp], sv[B], c0[B], az[B], af[B][kColUp];
      int cl[B];
#pragma unroll
      for (int b = 0; b < B; b++) {
        cl[b] = 0;
        sv[b] = T(0);
#pragma unroll
        for (int u = 0; u < kColUp; u++) in[b][u] = T(0);
        if (b < kn && active) {
          const int kk = kb + b;
          const int k = sz >= 0 ? kk : nz - 1 - kk;
          const int i = k * nxy + c;
          cl[b] = K.ccls[i];
          sv[b] = iso ? src[(size_t)i * G + g] : src[((size_t)i * G + g) * M + m];
#pragma unroll
          for (int u = 0; u < kColUp; u++)
            if (fu[u] >= 0) {
              if (cu[u] >= 0) in[b][u] = __ldcg(psi + ((size_t)(cu[u] + k * nxy) * G + g) * M + m);
              else if (bnd) in[b][u] = bnd_val(A, bnd, A.rslot[(size_t)fu[u] * n + i], g, m);
            }
        }
      }
#pragma unroll
      for (int b = 0; b < B; b++) {
        c0[b] = az[b] = T(0);
#pragma unroll
        for (int u = 0; u < kColUp; u++) af[b][u] = T(0);
        if (b < kn && active) {
          const T* cf = coef + (((size_t)cl[b] * G + g) * M + m) * (1 + F);
          c0[b] = cf[0];
#pragma unroll
          for (int u = 0; u < kColUp; u++)
            if (fu[u] >= 0) af[b][u] = cf[1 + fu[u]];
          if (fz >= 0) az[b] = cf[1 + fz];
        }
      }
#pragma unroll
      for (int b = 0; b < B; b++) {
        if (b >= kn) break;
        const int kk = kb + b;
        const int k = sz >= 0 ? kk : nz - 1 - kk;
        const int i = k * nxy + c;
        T v = T(0);
        if (active) {
          v = c0[b] * sv[b];
#pragma unroll
          for (int u = 0; u < kColUp; u++)
            if (af[b][u] != T(0)) v += af[b][u] * in[b][u];
          if (az[b] != T(0)) {
            if (kk > 0) v += az[b] * prev;
            else if (bnd) v += az[b] * bnd_val(A, bnd, A.rslot[(size_t)fz * n + i], g, m);
          }
          psi[((size_t)i * G + g) * M + m] = v;
        }
        prev = v;
        s_mom[wid][b][lane] = wm * v;
      }
      // publish the batch: the warp barrier orders every lane's psi stores before lane
      // 0's release
      __syncwarp();
      if (lane == 0) st_release_gpu64(prog + c, ep | (unsigned long long)(kb + kn));
      // the batch's moments: lane (layer b, group gl) sums its segment in direction order
      if (mom)
        for (int r = lane; r < kn * gn; r += 32) {
          const int b = r / gn, gg = r - b * gn;
          const int kk = kb + b;
          const int i = (sz >= 0 ? kk : nz - 1 - kk) * nxy + c;
          T acc = T(0);
          for (int dj = 0; dj < ndp; dj++) acc += s_mom[wid][b][gg * K.nd + dj];
          mom[((size_t)p * n + i) * G + g0 + gg] = acc;
        }
      __syncwarp();
    }
  }
}

// phi0[r] = sum over the sweep patterns of their moments, in pattern order.
template <typename T>
__global__ void k_mom_reduce(long long rows, int npat, const T* __restrict__ mom, T* phi0) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
    T s = T(0);
    for (int p = 0; p < npat; p++) s += mom[(size_t)p * rows + r];
    phi0[r] = s;
  }
}

// Per-class sweep coefficients (rd, a_x, a_y, a_z) for every (class, group, direction),
// evaluated on a representative cell of the class with the same diagonal as k_sweep_rden.
template <typename T>
__global__ void k_sweep_coef(SNOp<T> A, SweepFaces<T> W, int ncls, const int* __restrict__ rep, T* coef) {
  const int G = A.G, M = A.M;
  const long long N = (long long)ncls * G * M;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < N; r += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(r % M);
    const int cg = (int)(r / M);
    const int c = cg / G, g = cg - c * G;
    const int i = rep[c];
    const T rd = T(1) / sweep_den(A, W, i, g, m);
    coef[r * 4] = rd;
    // inflow face of axis a: the -a face when Omega_a > 0, the +a face otherwise
    const int fminus[3] = {3, 0, 4}, fplus[3] = {1, 2, 5};
    for (int a = 0; a < 3; a++) {
      const int f = A.dirs[(size_t)m * 3 + a] > T(0) ? fminus[a] : fplus[a];
      const T mu = sweep_mu(A, W, f, i, m);
      coef[r * 4 + 1 + a] = -(mu * W.win[(size_t)f * A.n + i]) * rd;
    }
  }
}

// Per-class coefficients of the level-set sweep (any mesh with a table of face normals):
// for class c, group g, direction m the row [rd, a_0 .. a_{F-1}] with rd = 1 / diagonal
// and a_f = -(mu_f w_in,f) rd on inflow faces that carry a flux in (interior, reflective),
// 0 on outflow, vacuum and absent faces; psi = rd src + sum_f a_f psi_in,f.
template <typename T>
__global__ void k_sweep_coef_faces(SNOp<T> A, SweepFaces<T> W, int ncls, const int* __restrict__ rep, T* coef) {
  const int G = A.G, M = A.M, F = A.F;
  const long long N = (long long)ncls * G * M;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < N; r += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(r % M);
    const int cg = (int)(r / M);
    const int c = cg / G, g = cg - c * G;
    const int i = rep[c];
    const T rd = T(1) / sweep_den(A, W, i, g, m);
    T* row = coef + r * (1 + F);
    row[0] = rd;
    for (int f = 0; f < F; f++) {
      T a = T(0);
      if (f < A.nf[i]) {
        const size_t o = (size_t)f * A.n + i;
        const T mu = sweep_mu(A, W, f, i, m);
        const int kd = A.kind[o];
        if (!(mu > T(0)) && (kd == PGPU_FACE_INTERIOR || kd == PGPU_FACE_REFLECTIVE)) a = -(mu * W.win[o]) * rd;
      }
      row[1 + f] = a;
    }
  }
}

// One level of the sweep for every pattern, coefficients from the per-class table: a row
// reads its cell's class, then per face one coefficient and, on an inflow face, the
// upwind angular flux (or the reflective inflow).  Same sums as k_sweep_level with the
// reciprocal diagonal distributed over the terms.
template <typename T>
__global__ void k_sweep_level_cls(SNOp<T> A, const unsigned short* __restrict__ ccls, const T* __restrict__ coef,
                                  int level, const int* __restrict__ pat_dirs_ptr, const int* __restrict__ pat_dirs,
                                  const int* __restrict__ pat_lev_ptr, const int* __restrict__ pat_nlev,
                                  const int* __restrict__ lev_ptr, const int* __restrict__ order,
                                  const SweepPtrs* __restrict__ P, int iso) {
  const int p = blockIdx.y;
  if (level >= pat_nlev[p]) return;
  const T* __restrict__ src = static_cast<const T*>(P->src);
  const T* __restrict__ bnd = static_cast<const T*>(P->bnd);
  T* psi = static_cast<T*>(P->psi);
  const int d0 = pat_dirs_ptr[p], nd = pat_dirs_ptr[p + 1] - d0;
  const int* lp = lev_ptr + pat_lev_ptr[p];
  const int c0 = lp[level], nc = lp[level + 1] - c0;
  const int* ord = order + (size_t)p * A.n;
  const int G = A.G, M = A.M, n = A.n, F = A.F;
  const int items = nc * G * nd;  // < 2^31 (checked at setup)
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < items; it += gridDim.x * blockDim.x) {
    const int rest = it / nd;
    const int di = it - rest * nd;
    const int ci = rest / G;
    const int g = rest - ci * G;
    const int i = ord[c0 + ci];
    const int m = pat_dirs[d0 + di];
    const size_t l = ((size_t)i * G + g) * M + m;
    const T* cf = coef + (((size_t)ccls[i] * G + g) * M + m) * (1 + F);
    T v = cf[0] * (iso ? src[(size_t)i * G + g] : src[l]);
    const int nfi = A.nf[i];
    for (int f = 0; f < nfi; f++) {
      const T a = cf[1 + f];
      if (a == T(0)) continue;
      const size_t o = (size_t)f * n + i;
      const int nb = A.nbr[o];
      if (nb >= 0) v += a * psi[((size_t)nb * G + g) * M + m];
      else if (bnd) v += a * bnd_val(A, bnd, A.rslot[o], g, m);
    }
    psi[l] = v;
  }
}

// phi0[i,g] = sum_m w_m psi[i,g,m] (one warp per (i,g) row, fixed order within the warp).
template <typename T>
__global__ void k_moment(int rows, int M, const T* __restrict__ w, const T* __restrict__ psi, T* phi0) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = warp; r < rows; r += nwarps) {
    T s = T(0);
    for (int m = lane; m < M; m += 32) s += w[m] * psi[r * M + m];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) phi0[r] = s;
  }
}

// Isotropic source q[i,g] = V sum_g2 (sigma_s(g2->g) + lam_s chi_g nu_sigma_f(g2)) phi0[i,g2]
// (+ b[i,g] when given).  lam_s is the Wielandt shift (0 for plain power iteration).
template <typename T>
__global__ void k_scatter_source(SNOp<T> A, const T* __restrict__ phi0, const T* __restrict__ b, T* q,
                                 double lam_val, const double* __restrict__ lam_dev) {
  const int G = A.G;
  const double lam_s = lam_dev ? *lam_dev : lam_val;  // the solve's current shift, or a given factor
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n * G; r += gridDim.x * blockDim.x) {
    const int i = r / G, g = r - i * G;
    const int mt = A.mat[i];
    const T* ssm = A.ss + (size_t)mt * G * G;
    T s = T(0);
    for (int g2 = 0; g2 < G; g2++) s += ssm[g2 * G + g] * phi0[(size_t)i * G + g2];
    if (lam_s != 0.0) {
      const T* ns = A.nsf + (size_t)mt * G;
      T f = T(0);
      for (int g2 = 0; g2 < G; g2++) f += ns[g2] * phi0[(size_t)i * G + g2];
      s += (T)lam_s * A.chi[(size_t)mt * G + g] * f;
    }
    s *= A.vol[i];
    if (b) s += b[r];
    q[r] = s;
  }
}

// Angular source q[i,g,m] = V sum_g2 sigma_s(g2->g) phi0[i,g2] (isotropic, broadcast over m).
template <typename T>
__global__ void k_broadcast(int rows, int M, const T* __restrict__ qi, T* qa) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < (long long)rows * M;
       l += (long long)gridDim.x * blockDim.x)
    qa[l] = qi[l / M];
}

// Incoming angular flux at reflective faces from the current psi: for slot s (cell i,
// face f, axis a) and its k-th incoming direction m, bnd[s,g,k] = psi[i,g,refl(m,a)].
template <typename T>
__global__ void k_reflect_extract(SNOp<T> A, int nrefl, const int* __restrict__ slot_cell,
                                  const int* __restrict__ slot_face, const T* __restrict__ psi, T* bnd) {
  const int G = A.G, M = A.M, Mh = A.Mh;
  const long long total = (long long)nrefl * G * Mh;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < total;
       l += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(l % Mh);
    const long long rest = l / Mh;
    const int g = (int)(rest % G);
    const int s = (int)(rest / G);
    const int m = A.klist[A.rkind[s] * Mh + k];
    T v = T(0);
    if (m >= 0) {
      const int i = slot_cell[s], f = slot_face[s];
      v = psi[((size_t)i * G + g) * M + A.refl[m * 3 + A.raxis[(size_t)f * A.n + i]]];
    }
    bnd[l] = v;
  }
}

// Exact matrix-free R psi (needs phi0 of the same psi).
template <typename T>
__global__ void k_apply_R(SNOp<T> A, const T* __restrict__ psi, const T* __restrict__ phi0, T* y) {
  const int G = A.G, M = A.M;
  const long long N = (long long)A.n * G * M;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(l % M);
    const long long r = l / M;
    const int g = (int)(r % G);
    const int i = (int)(r / G);
    const int mt = A.mat[i];
    const T V = A.vol[i];
    const T pl = psi[l];
    T acc = A.st[(size_t)mt * G + g] * V * pl;
    const T* ssm = A.ss + (size_t)mt * G * G;
    T sc = T(0);
    for (int g2 = 0; g2 < G; g2++) sc += ssm[g2 * G + g] * phi0[(size_t)i * G + g2];
    acc -= V * sc;
    const int nfi = A.nf[i];
    for (int f = 0; f < nfi; f++) {
      const size_t o = (size_t)f * A.n + i;
      const int kd = A.kind[o];
      const T mu = mu_of(A, f, i, m);
      const T muA = mu * A.area[o];
      if (kd == PGPU_FACE_INTERIOR) {
        const T* c = A.gauss + o * 4;
        const int j = A.nbr[o];
        const T pj = psi[((size_t)j * G + g) * M + m];
        if (mu > T(0)) acc += c[0] * muA * pl + c[1] * muA * pj;
        else acc += c[2] * muA * pl + c[3] * muA * pj;
      } else if (kd == PGPU_FACE_VACUUM) {
        if (mu > T(0)) {
          acc += muA * pl;
          if (A.use_ls) {
            const T* wl = A.lsw + o * A.F;
            for (int f2 = 0; f2 < nfi; f2++) {
              const int j = A.nbr[(size_t)f2 * A.n + i];
              if (A.kind[(size_t)f2 * A.n + i] == PGPU_FACE_INTERIOR)
                acc += wl[f2] * muA * (psi[((size_t)j * G + g) * M + m] - pl);
            }
          }
        }
      } else if (kd == PGPU_FACE_REFLECTIVE) {
        if (mu > T(0)) acc += muA * pl;
        else acc += muA * psi[((size_t)i * G + g) * M + A.refl[m * 3 + A.raxis[o]]];
      }
    }
    y[l] = acc;
  }
}

// ---- small vector kernels (deterministic reductions) ----

// x -= sum_k h[k] V[k]   (h on device)
template <typename T>
__global__ void k_sub_many(long long N, const T* __restrict__ V, long long ld, int nv, const double* __restrict__ h, T* x) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    T s = x[l];
    for (int k = 0; k < nv; k++) s -= (T)h[k] * V[(size_t)k * ld + l];
    x[l] = s;
  }
}

// Gram-Schmidt passes of the GMRES Arnoldi step over nv <= kGsMax basis vectors V_k
// (stride ld).  Element arithmetic is in the vectors' precision (FP32 for the mixed-
// precision correction solve: GB300's FP64 rate is 1/64 of FP32), reductions in FP64.  Products: each block row (blockIdx.y) takes kGsChunk vectors, so w is
// read once per chunk instead of once per vector, with few registers per thread.
constexpr int kGsMax = 32;
constexpr int kGsChunk = 8;
constexpr double kReorth = 0.5;  // second Gram-Schmidt pass when ||w|| drops below this share

// Decides on the device whether the Arnoldi step needs the second Gram-Schmidt pass:
// ||w|| after the first pass (*hn) below kReorth of its norm before (sqrt(*ww)).  *gate
// = 1 runs the gated second-pass kernels; otherwise h2 is zeroed, so the host adds
// nothing, and the step needs no host round trip between the passes.
__global__ void k_gs_gate(const double* ww, const double* hn, double* gate, double* h2, int nh) {
  const bool need = !(*hn >= kReorth * sqrt(fmax(*ww, 0.0)));
  *gate = need ? 1.0 : 0.0;
  if (!need)
    for (int k = 0; k < nh; k++) h2[k] = 0.0;
}

// Device-side state of one GMRES cycle run as a graph of conditional Arnoldi steps: the
// Hessenberg columns (rotated), the Givens rotations, the rotated right-hand side g and
// the cycle's progress.
struct ArnoldiState {
  double H[(kGsMax + 1) * kGsMax];  // column j at H + j (m + 1)
  double cs[kGsMax], sn[kGsMax], g[kGsMax + 1];
  double tol, res;
  int j;          // columns kept in this cycle
  int total;      // Arnoldi steps of the GMRES call so far
  int max_it;
  int stop;       // the cycle ended (converged, breakdown, the step cap or a non-finite value)
  int nonfinite;
  int reorth;     // steps of this cycle that ran the second Gram-Schmidt pass
};

__global__ void k_arnoldi_init(ArnoldiState* S, double beta, double tol, int total, int max_it) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int k = 0; k <= kGsMax; k++) S->g[k] = 0.0;
  S->g[0] = beta;
  S->tol = tol;
  S->res = beta;
  S->j = 0;
  S->total = total;
  S->max_it = max_it;
  S->stop = 0;
  S->nonfinite = 0;
  S->reorth = 0;
}

// Arnoldi step j of an m-step cycle, after its Gram-Schmidt products: the new Hessenberg
// column (first pass h1, plus the second pass h2 when the gate ran it), the rotations of
// the earlier columns, a new rotation and the residual |g[j+1]|; then the condition of
// step j+1's graph node (when there is one): 1 while the cycle goes on, 0 once it stops.
// The later steps' conditions start each launch at 0, so they are all skipped.
__global__ void k_arnoldi_step(ArnoldiState* S, int j, int m, const double* __restrict__ h1,
                               const double* __restrict__ h2, const double* __restrict__ hn,
                               const double* __restrict__ gate, cudaGraphConditionalHandle next, int has_next) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* col = S->H + (size_t)j * (m + 1);
  const bool second = *gate != 0.0;
  for (int k = 0; k <= j; k++) col[k] = h1[k] + (second ? h2[k] : 0.0);
  if (second) S->reorth++;
  const double hnext = *hn;
  S->total++;
  col[j + 1] = hnext;
  for (int k = 0; k < j; k++) {
    const double a = S->cs[k] * col[k] + S->sn[k] * col[k + 1];
    const double b = -S->sn[k] * col[k] + S->cs[k] * col[k + 1];
    col[k] = a;
    col[k + 1] = b;
  }
  const double rr = hypot(col[j], col[j + 1]);
  bool stop = false;
  if (rr == 0.0 || !(rr == rr)) {
    stop = true;  // column j is not kept
    S->nonfinite = !(rr == rr);
  } else {
    S->cs[j] = col[j] / rr;
    S->sn[j] = col[j + 1] / rr;
    col[j] = rr;
    col[j + 1] = 0.0;
    S->g[j + 1] = -S->sn[j] * S->g[j];
    S->g[j] = S->cs[j] * S->g[j];
    S->res = fabs(S->g[j + 1]);
    S->j = j + 1;
    if (S->res <= S->tol || hnext == 0.0) stop = true;
  }
  if (S->total >= S->max_it || j + 1 >= m) stop = true;
  S->stop = stop ? 1 : 0;
  if (has_next) cudaGraphSetConditional(next, stop ? 0u : 1u);
}

// out[k] = <V_k, w> for k < nv; reduction slots of chunk y at partials + y*kGsChunk*kMaxBlocks.
// With a gate, the whole grid returns at once when *gate == 0.
template <typename T>
__global__ void k_gs_dot(long long N, const T* __restrict__ V, long long ld, int nv, const T* __restrict__ w,
                         double* out, double* partials, unsigned int* tickets, const double* gate) {
  if (gate && *gate == 0.0) return;
  const int k0 = blockIdx.y * kGsChunk;
  const int nk = min(kGsChunk, nv - k0);
  // per-thread sums in precision T (a few elements each), block and grid sums in FP64
  T part[kGsChunk];
#pragma unroll
  for (int k = 0; k < kGsChunk; k++) part[k] = T(0);
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    const T x = w[l];
#pragma unroll
    for (int k = 0; k < kGsChunk; k++)
      if (k < nk) part[k] += V[(size_t)(k0 + k) * ld + l] * x;
  }
  double acc[kGsChunk];
#pragma unroll
  for (int k = 0; k < kGsChunk; k++) acc[k] = (double)part[k];
  ReduceSlots<kGsChunk> slots{partials + (size_t)blockIdx.y * kGsChunk * kMaxBlocks, tickets + blockIdx.y};
  double tot[kGsChunk];
  if (block_reduce_last<kGsChunk>(acc, slots, tot, nk) && threadIdx.x == 0)
    for (int k = 0; k < nk; k++) out[k0 + k] = tot[k];
}

// w -= sum_k h[k] V_k, then *out = ||w|| (skipped when a gate holds 0)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_gs_sub_norm(long long N, const T* __restrict__ V, long long ld, int nv,
                                                         const double* __restrict__ h, T* w, double* out,
                                                         ReduceSlots<1> slots, const double* gate) {
  if (gate && *gate == 0.0) return;
  T part = T(0);
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    T s = w[l];
    for (int k = 0; k < nv; k++) s -= (T)h[k] * V[(size_t)k * ld + l];
    w[l] = s;
    part += s * s;
  }
  double acc[1] = {(double)part};
  double tot[1];
  if (block_reduce_last<1>(acc, slots, tot) && threadIdx.x == 0) *out = sqrt(tot[0]);
}

// x += sum_k y[k] V[k]
template <typename T>
__global__ void k_add_many(long long N, const T* __restrict__ V, long long ld, int nv, const double* __restrict__ y, T* x) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    T s = x[l];
    for (int k = 0; k < nv; k++) s += (T)y[k] * V[(size_t)k * ld + l];
    x[l] = s;
  }
}

template <typename T>
__global__ void k_scale_to(long long N, const T* __restrict__ a, const double* __restrict__ s, int inv, T* b) {
  const T f = (T)(inv ? 1.0 / *s : *s);
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    b[l] = a[l] * f;
}

// c = a - b
template <typename T>
__global__ void k_sub(long long N, const T* __restrict__ a, const T* __restrict__ b, T* c) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    c[l] = a[l] - b[l];
}

template <typename T>
__global__ void k_norm2(long long N, const T* __restrict__ x, double* out, ReduceSlots<1> slots) {
  double acc[1] = {0.0};
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    acc[0] += (double)x[l] * (double)x[l];
  double tot[1];
  if (block_reduce_last<1>(acc, slots, tot) && threadIdx.x == 0) *out = sqrt(tot[0]);
}

template <typename T>
__global__ void k_mul(long long N, T* a, double f) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    a[l] = (T)((double)a[l] * f);
}

template <typename T>
__global__ void k_fill(long long N, T* a, T v) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    a[l] = v;
}

// x (FP64) += u (precision T)
template <typename T>
__global__ void k_add_cast(long long N, const T* __restrict__ u, double* x) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    x[l] += (double)u[l];
}

// x += u
template <typename T>
__global__ void k_add(long long N, const T* __restrict__ u, T* x) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    x[l] += u[l];
}

template <typename S, typename D>
__global__ void k_cast(long long N, const S* __restrict__ a, D* b) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    b[l] = (D)a[l];
}

// ---- outer-iteration kernels (FP64 state) ----

// fs_i = V sum_g nu_sigma_f phi0; S = sum fs.  The inner solve of a (shifted) power
// iteration step maps a fission source of total 1 to y, so lambda = lam_s + 1/S and
// k = 1/lambda (lam_s = 0: k = S).
__global__ void k_sn_fission(int n, int G, const int* __restrict__ mat, const double* __restrict__ vol,
                             const double* __restrict__ nsf, const double* __restrict__ phi0, double* fs,
                             SNOuter* os, ReduceSlots<1> slots, double lam_s) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* ns = nsf + (size_t)mat[i] * G;
    double s = 0.0;
    for (int g = 0; g < G; g++) s += ns[g] * phi0[(size_t)i * G + g];
    s *= vol[i];
    fs[i] = s;
    acc[0] += s;
  }
  double tot[1];
  if (block_reduce_last<1>(acc, slots, tot) && threadIdx.x == 0) {
    os->S = tot[0];
    os->k = 1.0 / (lam_s + 1.0 / tot[0]);
    os->nonfinite = !(tot[0] == tot[0]) || tot[0] == 0.0;
  }
}

// normalise fs by S, change vs fs_old, b = chi fs (isotropic, per (i,g); total 1).
__global__ void k_sn_source(int n, int G, const int* __restrict__ mat, const double* __restrict__ chi,
                            double* fs, double* fs_old, double* b, SNOuter* os, ReduceSlots<2> slots) {
  const double invS = 1.0 / os->S, invk = 1.0;
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double f = fs[i] * invS;
    double d = f - fs_old[i];
    fs_old[i] = f;
    acc[0] += d * d;
    acc[1] += f * f;
    const double* ch = chi + (size_t)mat[i] * G;
    for (int g = 0; g < G; g++) b[(size_t)i * G + g] = ch[g] * f * invk;
  }
  double tot[2];
  if (block_reduce_last<2>(acc, slots, tot) && threadIdx.x == 0) os->change = sqrt(tot[0] / tot[1]);
}

__global__ void k_sn_power_norm(int n, int G, const int* __restrict__ mat, const double* __restrict__ vol,
                                const double* __restrict__ ksf, const double* __restrict__ phi0, SNOuter* os,
                                ReduceSlots<1> slots) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* ks = ksf + (size_t)mat[i] * G;
    for (int g = 0; g < G; g++) acc[0] += 4.0 * M_PI * phi0[(size_t)i * G + g] * ks[g] * vol[i];
  }
  double tot[1];
  if (block_reduce_last<1>(acc, slots, tot) && threadIdx.x == 0) os->p0 = tot[0];
}

// phi = 4 pi phi0 * power / p0 (SNSolver::calculateScalarFlux + normalizeScalarFlux), q, P.
__global__ void k_sn_power_fields(int n, int G, const int* __restrict__ mat, const double* __restrict__ vol,
                                  const double* __restrict__ ksf, const double* __restrict__ nsf,
                                  const double* __restrict__ phi0, double power, double rel_flush, double* phi,
                                  double* q, double* P, SNOuter* os, ReduceSlots<2> slots) {
  const double f = 4.0 * M_PI * power / os->p0;
  const double k = os->k;
  const double flush = rel_flush * __longlong_as_double((long long)os->amax_phi) * fabs(f);
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* ks = ksf + (size_t)mat[i] * G;
    const double* ns = nsf + (size_t)mat[i] * G;
    const double V = vol[i];
    double qi = 0.0, Pi = 0.0;
    for (int g = 0; g < G; g++) {
      double v = phi0[(size_t)i * G + g] * f;
      if (v < 0.0 && v >= -flush) v = 0.0;
      phi[(size_t)i * G + g] = v;
      if (v < 0.0) acc[1] += 1.0;
      qi += v * ks[g] * V;
      Pi += v * ns[g] * V / k;
    }
    q[i] = qi;
    P[i] = Pi;
    acc[0] += qi;
  }
  double tot[2];
  if (block_reduce_last<2>(acc, slots, tot) && threadIdx.x == 0) {
    os->total_power = tot[0];
    os->negatives = (int)tot[1];
  }
}

// psi *= power / (p0 / 4 pi)  (SNSolver::normalizeAngularFlux); counts negatives.
__global__ void k_sn_psi_norm(long long N, double* psi, double power, double rel_flush, SNOuter* os,
                              ReduceSlots<1> slots) {
  const double f = 4.0 * M_PI * power / os->p0;
  const double flush = rel_flush * __longlong_as_double((long long)os->amax_psi) * fabs(f);
  double acc[1] = {0.0};
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    double v = psi[l] * f;
    if (v < 0.0 && v >= -flush) v = 0.0;
    psi[l] = v;
    if (v < 0.0) acc[0] += 1.0;
  }
  double tot[1];
  if (block_reduce_last<1>(acc, slots, tot) && threadIdx.x == 0) os->negatives += (int)tot[0];
}

}  // namespace pgpu

// ---------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------

namespace pgpu {
namespace {

struct SlotMaps {
  std::vector<int> cell, face;
};

// Ids of distinct face normals (rounded to `scale`).  Face slot f of neighbouring cells
// usually has the same normal, so the last normal seen in each slot is checked before
// the map.
class NormalIds {
 public:
  NormalIds(int F, double scale) : scale_(scale), last_nr_(F), last_(F), last_id_(F, -1) {}
  int id(int f, const double* nr) {
    if (last_id_[f] >= 0 && nr[0] == last_nr_[f][0] && nr[1] == last_nr_[f][1] && nr[2] == last_nr_[f][2])
      return last_id_[f];
    const std::array<long long, 3> key{std::llround(nr[0] * scale_), std::llround(nr[1] * scale_),
                                       std::llround(nr[2] * scale_)};
    int id;
    if (last_id_[f] >= 0 && last_[f] == key) {
      id = last_id_[f];
    } else {
      auto it = ids_.find(key);
      id = it == ids_.end() ? ids_.emplace(key, (int)ids_.size()).first->second : it->second;
    }
    last_nr_[f] = {nr[0], nr[1], nr[2]};
    last_[f] = key;
    last_id_[f] = id;
    return id;
  }
  size_t size() const { return ids_.size(); }

 private:
  double scale_;
  std::map<std::array<long long, 3>, int> ids_;
  std::vector<std::array<double, 3>> last_nr_;
  std::vector<std::array<long long, 3>> last_;
  std::vector<int> last_id_;
};

// Sweep patterns and upwind level sets.  Directions are grouped by the sign of mu against
// every distinct face normal of the mesh (or against every face when the mesh has too
// many distinct normals); with `levels`, each group's dependency graph is ordered by
// Kahn's algorithm (the level-set sweep; the tiled dataflow sweep needs the patterns only).
int build_schedule(const pgpu_sn_operator* op, Schedule& S, bool levels) {
  const int n = op->num_cells, F = op->num_faces, M = op->num_dirs, G = op->num_groups;
  auto mu = [&](int f, int i, int m) {
    const double* nr = op->normals + ((size_t)f * n + i) * 3;
    const double* d = op->directions + (size_t)m * 3;
    return d[0] * nr[0] + d[1] * nr[1] + d[2] * nr[2];
  };
  // distinct normals of interior faces
  NormalIds normal_id(F, 1e9);
  std::vector<int> face_nid((size_t)F * n, -1);
  for (int i = 0; i < n; i++)
    for (int f = 0; f < op->num_cell_faces[i]; f++) {
      const size_t o = (size_t)f * n + i;
      if (op->face_kind[o] != PGPU_FACE_INTERIOR) continue;
      face_nid[o] = normal_id.id(f, op->normals + o * 3);
    }
  const bool by_normal = normal_id.size() <= 4096;
  std::vector<std::vector<double>> nvec(normal_id.size());
  for (int i = 0; i < n; i++)
    for (int f = 0; f < op->num_cell_faces[i]; f++) {
      const size_t o = (size_t)f * n + i;
      if (face_nid[o] >= 0 && nvec[face_nid[o]].empty())
        nvec[face_nid[o]] = {op->normals[o * 3], op->normals[o * 3 + 1], op->normals[o * 3 + 2]};
    }
  std::map<std::string, int> pat_of_key;
  std::vector<std::vector<int>> pat_dirs;
  for (int m = 0; m < M; m++) {
    std::string key;
    if (by_normal) {
      key.resize(nvec.size());
      const double* d = op->directions + (size_t)m * 3;
      for (size_t k = 0; k < nvec.size(); k++)
        key[k] = (d[0] * nvec[k][0] + d[1] * nvec[k][1] + d[2] * nvec[k][2]) < 0.0 ? '1' : '0';
    } else {
      key.resize((size_t)F * n, '0');
      for (int i = 0; i < n; i++)
        for (int f = 0; f < op->num_cell_faces[i]; f++)
          if (op->face_kind[(size_t)f * n + i] == PGPU_FACE_INTERIOR && mu(f, i, m) < 0.0) key[(size_t)f * n + i] = '1';
    }
    auto it = pat_of_key.find(key);
    if (it == pat_of_key.end()) {
      pat_of_key[key] = (int)pat_dirs.size();
      pat_dirs.push_back({m});
    } else {
      pat_dirs[it->second].push_back(m);
    }
  }
  S = Schedule();
  S.npat = (int)pat_dirs.size();
  S.pat_dirs_ptr.push_back(0);
  for (auto& v : pat_dirs) {
    for (int m : v) S.pat_dirs.push_back(m);
    S.pat_dirs_ptr.push_back((int)S.pat_dirs.size());
  }
  if (!levels) return PGPU_OK;
  S.order.resize((size_t)S.npat * n);
  std::vector<int> indeg(n), head(n + 1), adj;
  for (int p = 0; p < S.npat; p++) {
    const int m = pat_dirs[p][0];
    // edge i -> j when j has an inflow face (mu < 0) whose neighbour is i
    std::fill(head.begin(), head.end(), 0);
    std::fill(indeg.begin(), indeg.end(), 0);
    for (int j = 0; j < n; j++)
      for (int f = 0; f < op->num_cell_faces[j]; f++) {
        const size_t o = (size_t)f * n + j;
        if (op->face_kind[o] == PGPU_FACE_INTERIOR && mu(f, j, m) < 0.0) {
          head[op->neighbors[o] + 1]++;
          indeg[j]++;
        }
      }
    for (int i = 0; i < n; i++) head[i + 1] += head[i];
    adj.assign(head[n], 0);
    std::vector<int> fill(head.begin(), head.end() - 1);
    for (int j = 0; j < n; j++)
      for (int f = 0; f < op->num_cell_faces[j]; f++) {
        const size_t o = (size_t)f * n + j;
        if (op->face_kind[o] == PGPU_FACE_INTERIOR && mu(f, j, m) < 0.0) adj[fill[op->neighbors[o]]++] = j;
      }
    int* ord = S.order.data() + (size_t)p * n;
    int cnt = 0;
    for (int i = 0; i < n; i++)
      if (indeg[i] == 0) ord[cnt++] = i;
    S.pat_lev_ptr.push_back((int)S.lev_ptr.size());
    S.lev_ptr.push_back(0);
    int lo = 0;
    while (lo < cnt) {
      const int hi = cnt;
      for (int k = lo; k < hi; k++) {
        const int i = ord[k];
        for (int e = head[i]; e < head[i + 1]; e++)
          if (--indeg[adj[e]] == 0) ord[cnt++] = adj[e];
      }
      S.lev_ptr.push_back(hi);
      lo = hi;
    }
    if (cnt != n) return fail(PGPU_ERR_INVALID, "the upwind graph of a direction has a cycle; this mesh cannot be swept");
    S.pat_nlev.push_back((int)S.lev_ptr.size() - S.pat_lev_ptr.back() - 1);
  }
  S.nlev = 0;
  for (int v : S.pat_nlev) S.nlev = std::max(S.nlev, v);
  S.grid_x.assign(S.nlev, 1);
  for (int p = 0; p < S.npat; p++) {
    const int* lp = S.lev_ptr.data() + S.pat_lev_ptr[p];
    const long long nd = S.pat_dirs_ptr[p + 1] - S.pat_dirs_ptr[p];
    for (int L = 0; L < S.pat_nlev[p]; L++) {
      long long items = (long long)(lp[L + 1] - lp[L]) * nd * G;
      S.grid_x[L] = std::max(S.grid_x[L], grid_for(items));
    }
  }
  return PGPU_OK;
}

template <typename T>
SNOp<T> make_op(const SNData& d);

template <>
SNOp<double> make_op<double>(const SNData& d) {
  return SNOp<double>{d.n, d.G, d.M, d.F, d.use_ls, d.nf.as<int>(), d.kind.as<int>(), d.nbr.as<int>(),
                      d.area.as<double>(), d.nrm.as<double>(), d.gauss.as<double>(), d.raxis.as<int>(),
                      d.rslot.as<int>(), d.lsw.as<double>(), d.lsdiag.as<double>(), d.mat.as<int>(),
                      d.vol.as<double>(), d.dirs.as<double>(), d.w.as<double>(), d.refl.as<int>(),
                      d.st.as<double>(), d.ss.as<double>(), d.chi.as<double>(), d.nsf.as<double>(),
                      d.d_rkind.as<int>(), d.d_kmap.as<int>(), d.d_klist.as<int>(), d.Mh};
}

template <>
SNOp<float> make_op<float>(const SNData& d) {
  return SNOp<float>{d.n, d.G, d.M, d.F, d.use_ls, d.nf.as<int>(), d.kind.as<int>(), d.nbr.as<int>(),
                     d.area32.as<float>(), d.nrm32.as<float>(), d.gauss32.as<float>(), d.raxis.as<int>(),
                     d.rslot.as<int>(), d.lsw32.as<float>(), d.lsdiag32.as<float>(), d.mat.as<int>(),
                     d.vol32.as<float>(), d.dirs32.as<float>(), d.w32.as<float>(), d.refl.as<int>(),
                     d.st32.as<float>(), d.ss32.as<float>(), d.chi32.as<float>(), d.nsf32.as<float>(),
                     d.d_rkind.as<int>(), d.d_kmap.as<int>(), d.d_klist.as<int>(), d.Mh};
}

template <int NV>
ReduceSlots<NV> sn_slots(SNData& d) {
  return ReduceSlots<NV>{d.partials.as<double>(), d.ticket.as<unsigned int>()};
}

int make_fp32(pgpu_problem* p) {
  SNData& d = *p->sn;
  if (d.have32) return PGPU_OK;
  cudaStream_t s = p->stream;
  auto conv = [&](DevBuf& src, DevBuf& dst) -> int {
    if (!src.ptr) return PGPU_OK;
    const long long cnt = (long long)(src.bytes / 8);
    int st = dev_alloc(dst, (size_t)cnt * 4, &p->bytes, p->stream);
    if (st) return st;
    launch(p, k_cast<double, float>, grid_for(cnt), kThreads, s, cnt, src.as<double>(), dst.as<float>());
    return PGPU_OK;
  };
  int st;
  if ((st = conv(d.area, d.area32)) || (st = conv(d.nrm, d.nrm32)) || (st = conv(d.gauss, d.gauss32)) ||
      (st = conv(d.lsw, d.lsw32)) || (st = conv(d.lsdiag, d.lsdiag32)) || (st = conv(d.vol, d.vol32)) ||
      (st = conv(d.dirs, d.dirs32)) || (st = conv(d.w, d.w32)) || (st = conv(d.st, d.st32)) ||
      (st = conv(d.ss, d.ss32)) || (st = conv(d.chi, d.chi32)) || (st = conv(d.nsf, d.nsf32)) ||
      (st = conv(d.mutab, d.mutab32)) || (st = conv(d.wout, d.wout32)) || (st = conv(d.windiag, d.windiag32)) ||
      (st = conv(d.win, d.win32)))
    return st;
  PGPU_CUDA(cudaGetLastError());
  d.have32 = true;
  return PGPU_OK;
}

template <typename T>
SweepFaces<T> make_faces(const SNData& d);

template <>
SweepFaces<double> make_faces<double>(const SNData& d) {
  return SweepFaces<double>{d.use_tab ? d.cls.as<unsigned char>() : nullptr, d.mutab.as<double>(),
                            d.wout.as<double>(), d.windiag.as<double>(), d.win.as<double>(), d.upwind ? 1 : 0,
                            d.rden.as<double>()};
}

template <>
SweepFaces<float> make_faces<float>(const SNData& d) {
  return SweepFaces<float>{d.use_tab ? d.cls.as<unsigned char>() : nullptr, d.mutab32.as<float>(),
                           d.wout32.as<float>(), d.windiag32.as<float>(), d.win32.as<float>(), d.upwind ? 1 : 0,
                           d.rden32.as<float>()};
}

// Reciprocal sweep diagonals in precision T, computed on first use.
template <typename T>
int ensure_rden(pgpu_problem* p, const SNOp<T>& A) {
  SNData& d = *p->sn;
  DevBuf& buf = sizeof(T) == 8 ? d.rden : d.rden32;
  if (buf.ptr) return PGPU_OK;
  const long long N = (long long)d.n * d.G * d.M;
  SweepFaces<T> W = make_faces<T>(d);  // rden still null here
  int st = dev_alloc(buf, (size_t)N * sizeof(T), &p->bytes, p->stream);
  if (st) return st;
  launch(p, k_sweep_rden<T>, grid_for(N), kThreads, p->stream, A, W, buf.as<T>());
  PGPU_CUDA(cudaGetLastError());
  return PGPU_OK;
}

}  // namespace
}  // namespace pgpu

namespace pgpu {
namespace {


// Per-class sweep coefficients in precision T (dataflow sweep with cell classes), computed
// on first use.
template <typename T>
int ensure_coef(pgpu_problem* p, const SNOp<T>& A) {
  SNData& d = *p->sn;
  DevBuf& buf = sizeof(T) == 8 ? d.coef : d.coef32;
  if (buf.ptr) return PGPU_OK;
  const long long N = (long long)d.ncls * d.G * d.M;
  SweepFaces<T> W = make_faces<T>(d);
  int st = dev_alloc(buf, (size_t)N * 4 * sizeof(T), &p->bytes, p->stream);
  if (st) return st;
  launch(p, k_sweep_coef<T>, grid_for(N), kThreads, p->stream, A, W, d.ncls, (const int*)d.d_crep.as<int>(),
         buf.as<T>());
  PGPU_CUDA(cudaGetLastError());
  return PGPU_OK;
}

// Per-class level-sweep coefficients in precision T, computed on first use.
template <typename T>
int ensure_level_coef(pgpu_problem* p, const SNOp<T>& A) {
  SNData& d = *p->sn;
  DevBuf& buf = sizeof(T) == 8 ? d.coef : d.coef32;
  if (buf.ptr) return PGPU_OK;
  const long long N = (long long)d.ncls * d.G * d.M;
  SweepFaces<T> W = make_faces<T>(d);
  int st = dev_alloc(buf, (size_t)N * (1 + d.F) * sizeof(T), &p->bytes, p->stream);
  if (st) return st;
  launch(p, k_sweep_coef_faces<T>, grid_for(N), kThreads, p->stream, A, W, d.ncls, (const int*)d.d_crep.as<int>(),
         buf.as<T>());
  PGPU_CUDA(cudaGetLastError());
  return PGPU_OK;
}

// The dataflow sweep for the problem's tile shape runs on a persistent grid: every CTA
// that fits on the device at once, at most one per task.  flow_prepare sizes it (before
// the launch is captured in the sweep graph), flow_launch enqueues it.
template <typename T, bool kClass, int TX, int TY, int TZ>
int flow_prepare(SNData& d) {
  const int S = d.kba_nd * d.kba_gchunk;
  constexpr int nt = TileShape<TX, TY, TZ>::kThreads;
  const size_t smem = flow_smem_bytes<T>(TX, TY, TZ, S, d.kba_gchunk);
  const void* fn = (const void*)k_sweep_flow<T, kClass, TX, TY, TZ>;
  int dev = 0, sms = 0, per_sm = 0;
  if (smem > 48u * 1024u) PGPU_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PGPU_CUDA(cudaGetDevice(&dev));
  PGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, smem));
  if (per_sm < 1) return fail(PGPU_ERR_CUDA, "the dataflow sweep does not fit on an SM");
  // CTAs per SM of the persistent grid: all that fit, or PGPU_FLOW_CTAS{64,32} (measurement)
  const char* ce = std::getenv(sizeof(T) == 8 ? "PGPU_FLOW_CTAS64" : "PGPU_FLOW_CTAS32");
  if (ce && std::atoi(ce) > 0) per_sm = std::min(per_sm, std::atoi(ce));
  d.flow_grid[sizeof(T) == 8 ? 0 : 1] = std::min(d.kba_ntasks, sms * per_sm);
  return PGPU_OK;
}

template <typename T, bool kClass, int TX, int TY, int TZ>
void flow_launch(SNData& d, cudaStream_t s, const SNOp<T>& A, const SweepFaces<T>& W, const FlowGeom& K,
                 const SweepPtrs* P, int iso) {
  const int S = d.kba_nd * d.kba_gchunk, grid = d.flow_grid[sizeof(T) == 8 ? 0 : 1];
  constexpr int nt = TileShape<TX, TY, TZ>::kThreads;
  const size_t smem = flow_smem_bytes<T>(TX, TY, TZ, S, d.kba_gchunk);
  k_sweep_flow<T, kClass, TX, TY, TZ><<<grid, nt, smem, s>>>(A, W, K, P, iso);
}

template <typename T, bool kClass>
int flow_prepare(SNData& d) {
  return d.kba_t[0] == 8 ? flow_prepare<T, kClass, 8, 8, 4>(d) : flow_prepare<T, kClass, 4, 4, 4>(d);
}

template <typename T, bool kClass>
void flow_launch(SNData& d, cudaStream_t s, const SNOp<T>& A, const SweepFaces<T>& W, const FlowGeom& K,
                 const SweepPtrs* P, int iso) {
  if (d.kba_t[0] == 8)
    flow_launch<T, kClass, 8, 8, 4>(d, s, A, W, K, P, iso);
  else
    flow_launch<T, kClass, 4, 4, 4>(d, s, A, W, K, P, iso);
}

// Coefficient tables, the pointer block and the persistent grid of precision T's sweeps
// (allocated on first use, so before any capture of a sweep into a graph).
template <typename T>
int sweep_prepare(pgpu_problem* p, const SNOp<T>& A) {
  SNData& d = *p->sn;
  const bool cls = d.kba && d.ncls > 0;
  const bool level_cls = !d.kba && d.ncls > 0;  // level sets with per-class coefficients
  int rst = cls ? ensure_coef<T>(p, A) : (level_cls ? ensure_level_coef<T>(p, A) : ensure_rden<T>(p, A));
  if (rst) return rst;
  if (!d.sweep_ptrs.ptr && (rst = dev_alloc(d.sweep_ptrs, sizeof(SweepPtrs), &p->bytes, p->stream))) return rst;
  if (d.kba && !d.flow_grid[sizeof(T) == 8 ? 0 : 1] && (rst = cls ? flow_prepare<T, true>(d) : flow_prepare<T, false>(d)))
    return rst;
  if (d.col && !d.col_grid[sizeof(T) == 8 ? 0 : 1]) {
    // persistent grid of the column sweep: every CTA (four task warps) that fits at once
    int dev = 0, sms = 0, per_sm = 0;
    PGPU_CUDA(cudaGetDevice(&dev));
    PGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_col<T, kColBatch<T>()>, 128, 0));
    if (per_sm < 1) return fail(PGPU_ERR_CUDA, "the column sweep does not fit on an SM");
    d.col_grid[sizeof(T) == 8 ? 0 : 1] = std::max(1, std::min((d.col_ntasks + 3) / 4, sms * per_sm));
  }
  return PGPU_OK;
}

template <typename T>
int sweep(pgpu_problem* p, const SNOp<T>& A, const T* src, int iso, const T* bnd, T* psi, T* mom = nullptr) {
  SNData& d = *p->sn;
  const Schedule& S = d.sched;
  const bool cls = d.kba && d.ncls > 0;
  const bool level_cls = !d.kba && d.ncls > 0;  // level sets with per-class coefficients
  int rst = sweep_prepare<T>(p, A);
  if (rst) return rst;
  const SweepFaces<T> W = make_faces<T>(d);
  SweepPtrs* P = d.sweep_ptrs.as<SweepPtrs>();
  // the sweep's launches are captured once per (precision, source kind) and replayed; the
  // buffers of this sweep go through the device-side pointer block
  launch(p, k_set_sweep_ptrs, 1, 1, p->stream, P, (const void*)src, (const void*)bnd, (void*)psi,
         (void*)(d.kba || d.col ? mom : nullptr));
  const int nlaunch = d.kba || d.col ? 2 : S.nlev;
  auto enqueue = [&](cudaStream_t st) {
    if (d.kba) {
      const FlowGeom K{d.kba_nx, d.kba_ny, d.kba_ntx, d.kba_nty, d.kba_ntz, d.kba_npat, d.kba_nd, d.kba_ntasks, d.kba_gchunk, d.kba_nchunk,
                       d.d_tiles.as<int>(), d.d_pat_sign.as<int>(), d.d_fpat_dirs_ptr.as<int>(), d.d_fpat_dirs.as<int>(),
                       cls ? d.d_ccls.as<unsigned short>() : nullptr,
                       cls ? (sizeof(T) == 8 ? d.coef.ptr : d.coef32.ptr) : nullptr, d.d_tile_cls.as<int>(),
                       d.d_tile_ncls.as<int>(), d.d_cell_lcls.as<unsigned char>(), d.flow_sync.as<FlowSync>(),
                       d.flow_flags.as<unsigned int>(), d.d_task_order.as<int>(), d.flow_sleep,
                       d.trace_buf.as<unsigned long long>()};
      k_flow_begin<<<1, 1, 0, st>>>(K.sync);
      if (cls)
        flow_launch<T, true>(d, st, A, W, K, P, iso);
      else
        flow_launch<T, false>(d, st, A, W, K, P, iso);
    } else if (d.col) {
      const ColGeom K{d.col_nxy, d.col_nz, S.npat, d.col_nd, d.col_ntasks, d.col_gchunk, d.col_nchunk,
                      d.d_col_up.as<int>(), d.d_col_zm.as<int>(), d.d_col_zp.as<int>(), d.d_col_sz.as<int>(),
                      d.d_pat_dirs_ptr.as<int>(), d.d_pat_dirs.as<int>(), d.d_col_order.as<int>(),
                      d.d_ccls.as<unsigned short>(), d.flow_sync.as<FlowSync>(),
                      d.flow_flags.as<unsigned long long>(), d.flow_sleep};
      k_flow_begin<<<1, 1, 0, st>>>(K.sync);
      k_sweep_col<T, kColBatch<T>()><<<d.col_grid[sizeof(T) == 8 ? 0 : 1], 128, 0, st>>>(
          A, K, (const T*)(sizeof(T) == 8 ? d.coef.ptr : d.coef32.ptr), P, iso);
    } else {
      for (int L = 0; L < S.nlev; L++) {
        dim3 g(S.grid_x[L], S.npat);
        if (level_cls)
          k_sweep_level_cls<T><<<g, kThreads, 0, st>>>(
              A, d.d_ccls.as<unsigned short>(), (const T*)(sizeof(T) == 8 ? d.coef.ptr : d.coef32.ptr), L,
              d.d_pat_dirs_ptr.as<int>(), d.d_pat_dirs.as<int>(), d.d_pat_lev_ptr.as<int>(), d.d_pat_nlev.as<int>(),
              d.d_lev_ptr.as<int>(), d.d_order.as<int>(), P, iso);
        else
          k_sweep_level<T><<<g, kThreads, 0, st>>>(
              A, W, L, d.d_pat_dirs_ptr.as<int>(), d.d_pat_dirs.as<int>(), d.d_pat_lev_ptr.as<int>(),
              d.d_pat_nlev.as<int>(), d.d_lev_ptr.as<int>(), d.d_order.as<int>(), P, iso);
      }
    }
  };
  if (d.capturing) {
    // inside a graph being captured (the GMRES cycle): the kernels themselves, no nested
    // graph launch and no timing; the caller counts the sweeps that run
    enqueue(p->stream);
    p->launches += nlaunch;
    PGPU_CUDA(cudaGetLastError());
    return PGPU_OK;
  }
  cudaGraphExec_t& gx = d.sweep_graph[sizeof(T) == 8 ? 0 : 1][iso ? 1 : 0];
  if (!gx) {
    cudaGraph_t graph;
    PGPU_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    enqueue(p->stream);
    PGPU_CUDA(cudaStreamEndCapture(p->stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&gx, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      gx = nullptr;
      return fail(PGPU_ERR_CUDA, std::string("sweep graph instantiation: ") + cudaGetErrorString(e));
    }
  }
  cudaEvent_t e0;
  prof_begin(p, &e0);
  const bool traced = d.kba && d.trace_sweep == d.sweeps && d.trace_buf.ptr;
  if (traced) launch(p, k_put<unsigned int>, 1, 1, p->stream, &d.flow_sync.as<FlowSync>()->trace_on, 1u);
  PGPU_CUDA(cudaGraphLaunch(gx, p->stream));
  if (traced) {
    // measurement only: the timeline of this sweep to a file of [ntasks][5] unsigned 64-bit
    launch(p, k_put<unsigned int>, 1, 1, p->stream, &d.flow_sync.as<FlowSync>()->trace_on, 0u);
    std::vector<unsigned long long> tl((size_t)d.kba_ntasks * 5);
    PGPU_CUDA(cudaMemcpyAsync(tl.data(), d.trace_buf.ptr, tl.size() * 8, cudaMemcpyDeviceToHost, p->stream));
    PGPU_CUDA(cudaStreamSynchronize(p->stream));
    if (FILE* fh = std::fopen(d.trace_file.c_str(), "wb")) {
      std::fwrite(tl.data(), 8, tl.size(), fh);
      std::fclose(fh);
    }
  }
  p->launches += nlaunch;
  p->prof_name = d.kba ? "k_sweep_flow" : (d.col ? "k_sweep_col" : "k_sweep_level");
  // Algorithmic bytes of one sweep: psi written once and read once per cell-group-
  // direction update (2 s_v), the source read per cell-group (s_v, or s_v per update for
  // an angular source), the scalar-flux moment written per cell-group (s_v) and the
  // material id per cell-group (4 B).
  const double sv = (double)sizeof(T);
  const double N = (double)d.n * d.G * d.M, nG = (double)d.n * d.G;
  prof_end(p, e0, nlaunch, N * 2.0 * sv + nG * (2.0 * sv + 4.0) + (iso ? 0.0 : N * sv));
  PGPU_CUDA(cudaGetLastError());
  d.sweeps++;
  return PGPU_OK;
}

template <typename T>
T* psi_work(SNData& d) {
  return sizeof(T) == 8 ? (T*)d.psi.ptr : (T*)d.psi32.ptr;
}


// y = T(x; b): sweep driven by the scattering (+ lam_s-shifted fission, lam_s the solve's
// shift held on the device) source of x's phi0 part plus b, and the reflective inflow held
// in x's boundary part; returns [phi0' | inflow'].
template <typename T>
int phi_space_T(pgpu_problem* p, const SNOp<T>& A, const T* x, const T* b, T* y) {
  SNData& d = *p->sn;
  const int nG = d.n * d.G;
  T* q = d.scat.as<T>();
  T* psi = psi_work<T>(d);
  launch(p, k_scatter_source<T>, grid_for(nG), kThreads, p->stream, A, x, b, q, 0.0, (const double*)d.lam_dev.as<double>());
  int st;
  if (d.kba || d.col) {
    // the dataflow sweeps write per-pattern moments; they are summed in pattern order
    const int npat = d.kba ? d.kba_npat : d.sched.npat;
    if (!d.mom.ptr && (st = dev_alloc(d.mom, (size_t)npat * nG * sizeof(double), &p->bytes, p->stream))) return st;
    T* mom = d.mom.as<T>();
    if ((st = sweep<T>(p, A, q, 1, d.nrefl ? x + nG : nullptr, psi, mom))) return st;
    launch(p, k_mom_reduce<T>, grid_for(nG), kThreads, p->stream, (long long)nG, npat, (const T*)mom, y);
  } else {
    if ((st = sweep<T>(p, A, q, 1, d.nrefl ? x + nG : nullptr, psi))) return st;
    launch(p, k_moment<T>, grid_for((long long)nG * 32), kThreads, p->stream, nG, d.M, A.w, psi, y);
  }
  if (d.nrefl) {
    const long long nb = (long long)d.nrefl * d.G * d.Mh;
    launch(p, k_reflect_extract<T>, grid_for(nb), kThreads, p->stream, A, d.nrefl, d.d_slot_cell.as<int>(),
                                                                   d.d_slot_face.as<int>(), psi, y + nG);
  }
  PGPU_CUDA(cudaGetLastError());
  return PGPU_OK;
}

// y = R x (angular space), using tmp (>= n*G) for phi0.
template <typename T>
int apply_R(pgpu_problem* p, const SNOp<T>& A, const T* x, T* y, T* tmp_phi0) {
  SNData& d = *p->sn;
  const int nG = d.n * d.G;
  const long long N = (long long)nG * d.M;
  launch(p, k_moment<T>, grid_for((long long)nG * 32), kThreads, p->stream, nG, d.M, A.w, x, tmp_phi0);
  launch(p, k_apply_R<T>, grid_for(N), kThreads, p->stream, A, x, tmp_phi0, y);
  PGPU_CUDA(cudaGetLastError());
  return PGPU_OK;
}

int ensure_krylov(pgpu_problem* p, size_t len, int restart, int es) {
  SNData& d = *p->sn;
  if (d.basis_len == len && d.restart == restart && d.krylov_prec == es) return PGPU_OK;
  d.drop_arnoldi_graphs();  // they hold the buffers replaced here
  int st;
  if (!d.lam_dev.ptr) {
    if ((st = dev_alloc(d.lam_dev, sizeof(double), &p->bytes, p->stream))) return st;
    PGPU_CUDA(cudaMemsetAsync(d.lam_dev.ptr, 0, sizeof(double), p->stream));
  }
  if ((st = dev_alloc(d.basis, (size_t)(restart + 1) * len * es, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.wvec, len * es, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.xvec, len * es, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.rhs, len * es, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.tmp, len * es, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.partials, (size_t)(restart + 4) * kMaxBlocks * 8, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.ticket, (size_t)(restart + 4) * 4, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.hbuf, (size_t)4 * (restart + 4) * 8, &p->bytes, p->stream))) return st;
  if (d.hpin) cudaFreeHost(d.hpin);
  d.hpin = nullptr;
  PGPU_CUDA(cudaMallocHost(&d.hpin, (size_t)4 * (restart + 4) * 8));
  // the scattering source is used by FP64 residual sweeps and by correction sweeps in
  // either precision: size it for FP64
  if ((st = dev_alloc(d.scat, (size_t)d.n * d.G * 8, &p->bytes, p->stream))) return st;
  if ((st = dev_alloc(d.phtmp, (size_t)d.n * d.G * es, &p->bytes, p->stream))) return st;
  PGPU_CUDA(cudaMemsetAsync(d.ticket.ptr, 0, (size_t)(restart + 4) * 4, p->stream));
  d.basis_len = len;
  d.restart = restart;
  d.krylov_prec = es;
  return PGPU_OK;
}

// GMRES(m) with classical Gram-Schmidt and one re-orthogonalisation (CGS2) for the
// correction equation A d = r, d starting at zero.  applyA(v, w) computes w = A v.
// Stops when ||r - A d|| <= max(rtol ||r||, atol) or after max_it Arnoldi steps.
//
// A cycle's Arnoldi steps run from a CUDA graph of m conditional nodes, one per step,
// captured once per precision: each body holds the step's sweep, its Gram-Schmidt
// products and k_arnoldi_step, which applies the Givens rotations on the device and
// sets the graph's condition to 0 once the cycle stops, so the remaining steps are
// skipped.  The host reads the cycle's state once per cycle (instead of once per step)
// and solves the small triangular system.  With profiling or a traced sweep the steps are
// driven from the host one at a time instead (same arithmetic).
template <typename T, typename App>
int gmres(pgpu_problem* p, long long len, App applyA, const T* r, T* dvec, double rtol, double atol,
          int max_it, int* iters, double* res_out) {
  SNData& d = *p->sn;
  const int m = d.restart;
  cudaStream_t s = p->stream;
  T* V = d.basis.as<T>();
  T* w = d.wvec.as<T>();
  double* h1 = d.hbuf.as<double>();
  double* h2 = h1 + (m + 4);
  double* hn = h2 + (m + 4);
  double* yv = hn + (m + 4);
  double* gate = hn + 1;
  const int gx = grid_for(len);
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
  double* hp = d.hpin;  // pinned mirror of hbuf
  int total = 0, st;
  double res = 0.0, tol = 0.0;
  bool first = true;
  ReduceSlots<1> nslot{d.partials.as<double>() + (size_t)(m + 2) * kMaxBlocks, d.ticket.as<unsigned int>() + (m + 2)};
  if (m + 2 > kGsMax) return fail(PGPU_ERR_INVALID, "GMRES restart length above the Gram-Schmidt kernels' limit");
  const int prec = sizeof(T) == 8 ? 0 : 1;
  const bool graphs = !p->profile && d.trace_sweep < 0;
  // Gram-Schmidt of step j: w_{j+1} (in V) against V_0..V_j, then normalised
  auto gs_step = [&](int j) {
    T* wj = V + (size_t)(j + 1) * len;
    // classical Gram-Schmidt with re-orthogonalisation when needed ("twice is enough"):
    // h1 = V^T w (and <w, w>), w -= V h1 with its norm; a second pass only when the
    // norm fell below kReorth of the original (cancellation)
    // grids of 2 (products) and 4 (subtraction) CTAs per SM: FP64 issue bounds these kernels,
    // and fewer threads mean fewer per-thread reductions for the same products
    const dim3 gd1(std::min(gx, kMaxGrid / 4), (j + 2 + kGsChunk - 1) / kGsChunk);
    const dim3 gd(std::min(gx, kMaxGrid / 4), (j + 1 + kGsChunk - 1) / kGsChunk);
    const int gsub = std::min(gx, kMaxGrid / 2);
    double* part = d.partials.as<double>();
    unsigned int* tick = d.ticket.as<unsigned int>();
    launch(p, k_gs_dot<T>, gd1, kThreads, s, len, (const T*)V, len, j + 2, (const T*)wj, h1, part, tick,
           (const double*)nullptr);
    launch(p, k_gs_sub_norm<T>, gsub, kThreads, s, len, (const T*)V, len, j + 1, (const double*)h1, wj, hn, nslot,
           (const double*)nullptr);
    // the second pass, decided and (if needed) run on the device
    launch(p, k_gs_gate, 1, 1, s, (const double*)(h1 + j + 1), (const double*)hn, gate, h2, j + 1);
    launch(p, k_gs_dot<T>, gd, kThreads, s, len, (const T*)V, len, j + 1, (const T*)wj, h2, part, tick,
           (const double*)gate);
    launch(p, k_gs_sub_norm<T>, gsub, kThreads, s, len, (const T*)V, len, j + 1, (const double*)h2, wj, hn, nslot,
           (const double*)gate);
    launch(p, k_scale_to<T>, gx, kThreads, s, len, (const T*)wj, (const double*)hn, 1, wj);
  };
  // the cycle graph, captured on first use
  if (graphs && !d.arn_graph[prec]) {
    if (!d.arn.ptr && (st = dev_alloc(d.arn, sizeof(ArnoldiState), &p->bytes, s))) return st;
    ArnoldiState* AS = d.arn.as<ArnoldiState>();
    cudaGraph_t graph = nullptr;
    // one condition per step node (a condition belongs to one node): step 0's starts each
    // launch at 1, the others at 0 until the step before sets them
    std::vector<cudaGraphConditionalHandle> cond(m, 0);
    const long long counted = p->launches;
    int cst = PGPU_OK;
    auto ck = [&](cudaError_t e, const char* what) {
      if (cst == PGPU_OK && e != cudaSuccess)
        cst = fail(PGPU_ERR_CUDA, std::string("GMRES cycle graph, ") + what + ": " + cudaGetErrorString(e));
      return cst == PGPU_OK;
    };
    if (ck(cudaGraphCreate(&graph, 0), "create"))
      for (int j = 0; j < m; j++)
        if (!ck(cudaGraphConditionalHandleCreate(&cond[j], graph, j == 0 ? 1u : 0u, cudaGraphCondAssignDefault),
                "condition"))
          break;
    cudaGraphNode_t prev = nullptr;
    for (int j = 0; j < m && cst == PGPU_OK; j++) {
      cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
      cp.conditional.handle = cond[j];
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      if (!ck(cudaGraphAddNode(&node, graph, prev ? &prev : nullptr, nullptr, prev ? 1 : 0, &cp), "step node")) break;
      if (!ck(cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal),
              "capture"))
        break;
      d.capturing = true;
      const int ae = applyA(V + (size_t)j * len, V + (size_t)(j + 1) * len);
      gs_step(j);
      k_arnoldi_step<<<1, 1, 0, s>>>(AS, j, m, h1, h2, hn, gate, j + 1 < m ? cond[j + 1] : 0ull, j + 1 < m ? 1 : 0);
      d.capturing = false;
      cudaGraph_t body = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(s, &body);
      if (ae != PGPU_OK && cst == PGPU_OK) cst = ae;
      ck(ee, "end capture");
      ck(cudaGetLastError(), "step launches");
      prev = node;
    }
    if (cst == PGPU_OK) {
      d.arn_step_launches[prec] = (int)((p->launches - counted) / m) + 1;  // + k_arnoldi_step
      ck(cudaGraphInstantiate(&d.arn_graph[prec], graph, 0), "instantiate");
    }
    p->launches = counted;
    if (graph) cudaGraphDestroy(graph);
    if (cst != PGPU_OK) {
      d.arn_graph[prec] = nullptr;
      return cst;
    }
  }
  // a sweep that returned early after a bounded wait ran out leaves unfinished tiles;
  // report that cause rather than the NaN it may lead to
  auto nan_cause = [&]() -> int {
    if (d.kba || d.col) {
      unsigned int err = 0;
      if (int e = read_small(&err, &d.flow_sync.as<FlowSync>()->error, sizeof(err), s)) return e;
      if (err) return fail(PGPU_ERR_TIMEOUT, "sweep: a wait for an upwind tile ran out (kernel returned early)");
    }
    return fail(PGPU_ERR_NAN, "NaN in the transport correction solve");
  };
  PGPU_CUDA(cudaMemsetAsync(dvec, 0, len * sizeof(T), s));
  while (true) {
    if (first) {
      PGPU_CUDA(cudaMemcpyAsync(V, r, len * sizeof(T), cudaMemcpyDeviceToDevice, s));
    } else {
      if ((st = applyA(dvec, w))) return st;
      launch(p, k_sub<T>, gx, kThreads, s, len, r, (const T*)w, V);
    }
    launch(p, k_norm2<T>, gx, kThreads, s, len, (const T*)V, hn, nslot);
    double beta;
    if ((st = read_small(&beta, hn, 8, s))) return st;
    if (!(beta == beta)) return nan_cause();
    if (first) {
      tol = std::fmax(rtol * beta, atol);
      first = false;
    }
    res = beta;
    if (beta <= tol || total >= max_it) break;
    launch(p, k_scale_to<T>, gx, kThreads, s, len, (const T*)V, (const double*)hn, 1, V);
    int j = 0;
    if (graphs) {
      ArnoldiState* AS = d.arn.as<ArnoldiState>();
      launch(p, k_arnoldi_init, 1, 1, s, AS, beta, tol, total, max_it);
      PGPU_CUDA(cudaGraphLaunch(d.arn_graph[prec], s));
      ArnoldiState hs;
      if ((st = read_small(&hs, AS, sizeof(hs), s))) return st;
      const int steps = hs.total - total;
      d.sweeps += steps;  // one sweep per step
      p->launches += (long long)steps * d.arn_step_launches[prec];
      d.reorth += hs.reorth;
      total = hs.total;
      if (hs.nonfinite) return nan_cause();
      j = hs.j;
      res = hs.res;
      for (int c = 0; c < j; c++)
        for (int k = 0; k <= c; k++) H[(size_t)c * (m + 1) + k] = hs.H[(size_t)c * (m + 1) + k];
      for (int k = 0; k <= j; k++) g[k] = hs.g[k];
    } else {
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      for (; j < m && total < max_it; j++) {
        T* vj = V + (size_t)j * len;
        T* wj = V + (size_t)(j + 1) * len;  // the new vector is built in place
        if ((st = applyA(vj, wj))) return st;
        gs_step(j);
        PGPU_CUDA(cudaGetLastError());
        // h1, h2, ||w|| and the gate (adjacent in hbuf): one copy into pinned host memory
        PGPU_CUDA(cudaMemcpyAsync(hp, h1, (size_t)(2 * (m + 4) + 2) * 8, cudaMemcpyDeviceToHost, s));
        PGPU_CUDA(cudaStreamSynchronize(s));
        double hnext = hp[2 * (m + 4)];
        double* col = &H[(size_t)j * (m + 1)];
        for (int k = 0; k <= j; k++) col[k] = hp[k];
        if (hp[2 * (m + 4) + 1] != 0.0) {
          for (int k = 0; k <= j; k++) col[k] += hp[(m + 4) + k];
          d.reorth++;
        }
        total++;
        col[j + 1] = hnext;
        for (int k = 0; k < j; k++) {
          double a = cs[k] * col[k] + sn[k] * col[k + 1];
          double b = -sn[k] * col[k] + cs[k] * col[k + 1];
          col[k] = a;
          col[k + 1] = b;
        }
        double rr = std::hypot(col[j], col[j + 1]);
        if (rr == 0.0 || !(rr == rr)) break;
        cs[j] = col[j] / rr;
        sn[j] = col[j + 1] / rr;
        col[j] = rr;
        col[j + 1] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        res = std::fabs(g[j + 1]);
        if (res <= tol || hnext == 0.0) {
          j++;
          break;
        }
      }
    }
    if (j == 0) break;
    std::vector<double> y(j, 0.0);
    for (int k = j - 1; k >= 0; k--) {
      double t = g[k];
      for (int c = k + 1; c < j; c++) t -= H[(size_t)c * (m + 1) + k] * y[c];
      y[k] = t / H[(size_t)k * (m + 1) + k];
    }
    PGPU_CUDA(cudaMemcpyAsync(yv, y.data(), j * 8, cudaMemcpyHostToDevice, s));
    launch(p, k_add_many<T>, gx, kThreads, s, len, (const T*)V, len, j, (const double*)yv, dvec);
    PGPU_CUDA(cudaGetLastError());
    if (res <= tol || total >= max_it) break;
  }
  PGPU_CUDA(cudaStreamSynchronize(s));
  *iters = total;
  *res_out = res;
  return PGPU_OK;
}

template <typename T>
int norm_of(pgpu_problem* p, long long len, const T* x, double* out) {
  SNData& d = *p->sn;
  double* hn = d.hbuf.as<double>() + 3 * (d.restart + 4) + (d.restart + 2);
  ReduceSlots<1> slot{d.partials.as<double>() + (size_t)(d.restart + 3) * kMaxBlocks, d.ticket.as<unsigned int>() + (d.restart + 3)};
  launch(p, k_norm2<T>, grid_for(len), kThreads, p->stream, len, x, hn, slot);
  PGPU_CUDA(cudaMemcpyAsync(out, hn, 8, cudaMemcpyDeviceToHost, p->stream));
  PGPU_CUDA(cudaStreamSynchronize(p->stream));
  return PGPU_OK;
}

// Failure injection of the dataflow sweep's bounded wait (FlowSync::stall): the value of
// PGPU_DEBUG_SWEEP_STALL (a task index + 1), read at the start of every solve; unset or 0
// in normal use.
unsigned int debug_sweep_stall() {
  const char* e = std::getenv("PGPU_DEBUG_SWEEP_STALL");
  return e ? (unsigned int)std::strtoul(e, nullptr, 10) : 0u;
}

int read_outer(pgpu_problem* p, SNOuter& os) {
  SNData& d = *p->sn;
  FlowSync fs{0u, 0u, 0u, 0u};
  int st = read_small(&os, d.oscal.ptr, sizeof(os), p->stream);
  if (st == PGPU_OK && (d.kba || d.col)) st = read_small(&fs, d.flow_sync.ptr, sizeof(fs), p->stream);
  if (st) return st;
  if (fs.error) return fail(PGPU_ERR_TIMEOUT, "sweep: a wait for an upwind tile ran out (kernel returned early)");
  return PGPU_OK;
}

// Power iteration on R x = (1/k) F x.  The state x (FP64) is [phi0 | reflective inflow]
// in scalar-flux space or psi in angular space.  Every outer iteration evaluates the FP64
// residual of the inner system, solves the correction equation in precision T (FP64, or
// FP32 for mixed precision: iterative refinement), updates x, and renormalises the
// fission source.  The correction solve reduces the FP64 residual by kEta (measured on the
// S8 workload: 0.2 needs 419 sweeps per solve against 952 at 0.02 and 487 at 0.1, with the
// same outer count and k; 0.5 starts to cost outer iterations).
constexpr double kEta = 0.2;
// Wielandt shift: lambda_s = 1 / (k (1 + shift)) (options.shift) once at least kShiftAfter
// outer iterations have run and |dk| < kShiftWhenDk.  The inner operator I - T (S +
// lambda_s F) stays nonsingular while k (1 + shift) is above the fundamental k; the
// shifted iteration's dominance ratio is (1/k1 - lambda_s) / (1/k2 - lambda_s).
constexpr int kShiftAfter = 3;
constexpr double kShiftDefault = 0.05;  // relative shift of k (measured best on the S8 workload)
constexpr double kShiftMargin = 50.0;   // the shifted k is at least k + kShiftMargin |dk| (the estimate
                                        // lags the fundamental k by about dk rho / (1 - rho))
// |dk| below which the shift starts.  The margin already keeps an early shift weak, and
// waiting for |dk| < 1e-3 spent 21 unshifted outer iterations of the S8 workload's 37 on
// getting k to 1e-3: from 0.1, 28 outer iterations and 0.21 against 0.26 s per FP64 solve
// (mixed 0.155 against 0.19 s; hexagonal workload 6.14 against 6.31 s), same k to 1e-11.
constexpr double kShiftWhenDk = 0.1;

template <typename T>
int solve_T(pgpu_problem* p, const pgpu_options* opt, pgpu_stats* stats) {
  SNData& d = *p->sn;
  cudaStream_t s = p->stream;
  const int n = d.n, G = d.G, M = d.M, nG = n * G;
  const long long N = (long long)nG * M;
  const bool phi_space = d.upwind && !d.use_ls;
  const long long len = phi_space ? (long long)nG + (long long)d.nrefl * G * d.Mh : N;
  const int restart = 30;
  int st;
  if ((st = ensure_krylov(p, (size_t)len, restart, (int)sizeof(T)))) return st;
  if (d.x64.bytes < (size_t)len * 8) {
    if ((st = dev_alloc(d.x64, (size_t)len * 8, &p->bytes, p->stream)) || (st = dev_alloc(d.r64, (size_t)len * 8, &p->bytes, p->stream)) ||
        (st = dev_alloc(d.rhs64, (size_t)len * 8, &p->bytes, p->stream)))
      return st;
  }
  SNOp<T> A = make_op<T>(d);
  SNOp<double> A64 = make_op<double>(d);
  // everything the sweeps allocate on first use, before a GMRES cycle is captured
  if ((st = sweep_prepare<double>(p, A64)) || (st = sweep_prepare<T>(p, A))) return st;
  if (phi_space && (d.kba || d.col) && !d.mom.ptr &&
      (st = dev_alloc(d.mom, (size_t)(d.kba ? d.kba_npat : d.sched.npat) * nG * sizeof(double), &p->bytes, p->stream)))
    return st;
  SNOuter* dos = d.oscal.as<SNOuter>();
  double* x64 = d.x64.as<double>();
  double* r64 = d.r64.as<double>();
  double* rhs64 = d.rhs64.as<double>();
  T* rT = d.rhs.as<T>();    // correction right-hand side in precision T
  T* dT = d.tmp.as<T>();    // correction in precision T
  T* phT = d.phtmp.as<T>();
  double* bsrc = d.src.as<double>();  // isotropic fission source b = chi fs / k, [n*G]
  double* phi0 = d.phi0.as<double>();
  double* ph64 = d.phi.as<double>();  // FP64 scratch [n*G] until the final fields
  ReduceSlots<1> s1{d.partials.as<double>(), d.ticket.as<unsigned int>()};
  ReduceSlots<2> s2{d.partials.as<double>(), d.ticket.as<unsigned int>()};
  const int gl = grid_for(len), gn = grid_for(n), gG = grid_for(nG);
  d.sweeps = 0;

  cudaEvent_t e0, e1;
  PGPU_CUDA(cudaEventCreate(&e0));
  PGPU_CUDA(cudaEventCreate(&e1));
  PGPU_CUDA(cudaEventRecord(e0, s));

  // flat start: phi0 = 1; x = [1 | 0] or psi = 1; k = 1
  SNOuter init;
  std::memset(&init, 0, sizeof(init));
  init.k = 1.0;
  launch(p, k_put<SNOuter>, 1, 1, s, dos, init);
  if (d.kba || d.col) {
    PGPU_CUDA(cudaMemsetAsync(&d.flow_sync.as<FlowSync>()->error, 0, sizeof(unsigned int), s));
    launch(p, k_put<unsigned int>, 1, 1, s, &d.flow_sync.as<FlowSync>()->stall, debug_sweep_stall());
  }
  launch(p, k_fill<double>, gG, kThreads, s, (long long)nG, phi0, 1.0);
  PGPU_CUDA(cudaMemsetAsync(x64, 0, len * 8, s));
  launch(p, k_fill<double>, grid_for(phi_space ? nG : N), kThreads, s, phi_space ? (long long)nG : N, x64, 1.0);
  launch(p, k_sn_fission, gn, kThreads, s, n, G, (const int*)d.mat.as<int>(), (const double*)d.vol.as<double>(),
         (const double*)d.nsf.as<double>(), (const double*)phi0, d.fs.as<double>(), dos, s1, 0.0);
  SNOuter os;
  if ((st = read_outer(p, os))) return st;
  if (os.nonfinite || os.S <= 0.0) return fail(PGPU_ERR_INVALID, "no fission source in the initial flux");
  os.k = 1.0;
  launch(p, k_put<SNOuter>, 1, 1, s, dos, os);
  PGPU_CUDA(cudaMemsetAsync(d.fs_old.ptr, 0, (size_t)n * 8, s));
  launch(p, k_sn_source, gn, kThreads, s, n, G, (const int*)d.mat.as<int>(), (const double*)d.chi.as<double>(),
         d.fs.as<double>(), d.fs_old.as<double>(), bsrc, dos, s2);
  launch(p, k_scale_to<double>, gl, kThreads, s, len, (const double*)x64, (const double*)&dos->S, 1, x64);
  PGPU_CUDA(cudaGetLastError());

  // Wielandt shift lam_s = 1/(k (1 + shift)), switched on once k has settled (scalar-flux
  // space only); 0 means plain power iteration.  The sweeps' sources read it on the device.
  double lam_s = 0.0;
  const char* swe = std::getenv("PGPU_SN_SHIFT_WHEN_DK");  // measurement override of kShiftWhenDk
  const double shift_when_dk = swe ? std::atof(swe) : kShiftWhenDk;
  const char* sae = std::getenv("PGPU_SN_SHIFT_AFTER");  // measurement override of kShiftAfter
  const int shift_after = sae ? std::atoi(sae) : kShiftAfter;
  const char* ete = std::getenv("PGPU_SN_ETA");  // measurement override of kEta
  const double eta = ete ? std::atof(ete) : kEta;
  launch(p, k_put<double>, 1, 1, s, d.lam_dev.as<double>(), 0.0);

  // correction operators in precision T
  T* zT = psi_work<T>(d);
  auto applyA = [&](const T* v, T* w) -> int {
    int e;
    if (phi_space) {
      if ((e = phi_space_T<T>(p, A, v, nullptr, w))) return e;  // w = T (S + lam_s F) v
      launch(p, k_sub<T>, gl, kThreads, s, len, v, (const T*)w, w);  // w = v - T_s v
      return PGPU_OK;
    }
    if ((e = sweep<T>(p, A, v, 0, nullptr, zT))) return e;  // z = P^-1 v
    return apply_R<T>(p, A, zT, w, phT);                     // w = R z
  };

  int outer = 0, inner_total = 0;
  double change = 1.0, dk = 1.0, k_prev = 1.0, res = 0.0;
  bool converged = false;
  for (outer = 1; outer <= opt->max_outer; outer++) {
    // initial guess of the inner solution: an eigenvector x with fission total 1 maps to
    // x / (lambda - lam_s)
    launch(p, k_mul<double>, gl, kThreads, s, len, x64, 1.0 / (1.0 / k_prev - lam_s));
    // FP64 residual of the inner system for the current fission source
    double scale = 0.0;
    if (phi_space) {
      if ((st = phi_space_T<double>(p, A64, x64, bsrc, r64))) return st;  // T((S + lam_s F) x + b)
      launch(p, k_sub<double>, gl, kThreads, s, len, (const double*)r64, (const double*)x64, r64);
      if ((st = norm_of<double>(p, len, x64, &scale))) return st;
    } else {
      launch(p, k_broadcast<double>, grid_for(N), kThreads, s, nG, M, (const double*)bsrc, rhs64);
      if ((st = apply_R<double>(p, A64, x64, r64, ph64))) return st;
      launch(p, k_sub<double>, gl, kThreads, s, len, (const double*)rhs64, (const double*)r64, r64);
      if ((st = norm_of<double>(p, len, rhs64, &scale))) return st;
    }
    double rnorm = 0.0;
    if ((st = norm_of<double>(p, len, r64, &rnorm))) return st;
    int it = 0;
    const double atol = 1e-14 * scale;
    if (rnorm > atol) {
      const T* rin;
      if (sizeof(T) == 8) {
        rin = (const T*)r64;
      } else {
        launch(p, k_cast<double, T>, gl, kThreads, s, len, (const double*)r64, rT);
        rin = rT;
      }
      if ((st = gmres<T>(p, len, applyA, rin, dT, eta, sizeof(T) == 8 ? atol : 0.0, opt->max_inner, &it, &res))) return st;
      if (phi_space) {
        launch(p, k_add_cast<T>, gl, kThreads, s, len, (const T*)dT, x64);
      } else {
        if ((st = sweep<T>(p, A, dT, 0, nullptr, zT))) return st;  // x += P^-1 d
        launch(p, k_add_cast<T>, gl, kThreads, s, len, (const T*)zT, x64);
      }
    }
    inner_total += it;
    // fission source, k and normalisation (FP64)
    if (phi_space) {
      PGPU_CUDA(cudaMemcpyAsync(phi0, x64, (size_t)nG * 8, cudaMemcpyDeviceToDevice, s));
    } else {
      launch(p, k_moment<double>, grid_for((long long)nG * 32), kThreads, s, nG, M, (const double*)d.w.as<double>(),
             (const double*)x64, phi0);
    }
    launch(p, k_sn_fission, gn, kThreads, s, n, G, (const int*)d.mat.as<int>(), (const double*)d.vol.as<double>(),
           (const double*)d.nsf.as<double>(), (const double*)phi0, d.fs.as<double>(), dos, s1, lam_s);
    launch(p, k_scale_to<double>, gl, kThreads, s, len, (const double*)x64, (const double*)&dos->S, 1, x64);
    launch(p, k_sn_source, gn, kThreads, s, n, G, (const int*)d.mat.as<int>(), (const double*)d.chi.as<double>(),
           d.fs.as<double>(), d.fs_old.as<double>(), bsrc, dos, s2);
    PGPU_CUDA(cudaGetLastError());
    if ((st = read_outer(p, os))) return st;
    if (os.nonfinite || !(os.k == os.k) || !(os.k > 0.0)) return fail(PGPU_ERR_NAN, "non-finite fission source");
    change = os.change;
    dk = std::fabs(os.k - k_prev);
    k_prev = os.k;
    if (opt->verbose)
      std::printf("pgpu sn outer %d: k = %.12f  dk = %.3e  source change = %.3e  |r|/scale = %.2e  gmres = %d  lam_s = %.6f\n",
                  outer, os.k, dk, change, scale > 0 ? rnorm / scale : 0.0, it, lam_s);
    if (dk < opt->tol_k && change < opt->tol_flux) {
      converged = true;
      break;
    }
    const double sh = opt->shift < 0.0 ? kShiftDefault : opt->shift;
    if (phi_space && outer >= shift_after && dk < shift_when_dk && sh > 0.0) {
      lam_s = 1.0 / std::fmax(os.k * (1.0 + sh), os.k + kShiftMargin * dk);  // above the fundamental k
      launch(p, k_put<double>, 1, 1, s, d.lam_dev.as<double>(), lam_s);
    }
  }

  // psi in FP64 from the converged state (one more sweep in scalar-flux space)
  double* psi = d.psi.as<double>();
  if (phi_space) {
    // source of the eigen-equation: (S + F / k) phi0
    launch(p, k_scatter_source<double>, gG, kThreads, s, A64, (const double*)x64, (const double*)nullptr, ph64,
           1.0 / k_prev, (const double*)nullptr);
    if ((st = sweep<double>(p, A64, ph64, 1, d.nrefl ? x64 + nG : nullptr, psi))) return st;
  } else {
    PGPU_CUDA(cudaMemcpyAsync(psi, x64, (size_t)N * 8, cudaMemcpyDeviceToDevice, s));
  }
  launch(p, k_moment<double>, grid_for((long long)nG * 32), kThreads, s, nG, M, (const double*)d.w.as<double>(),
         (const double*)psi, phi0);
  PGPU_CUDA(cudaMemsetAsync(&dos->amax_phi, 0, 2 * sizeof(unsigned long long), s));
  launch(p, k_absmax<double>, gG, kThreads, s, (long long)nG, (const double*)phi0, &dos->amax_phi);
  launch(p, k_absmax<double>, grid_for(N), kThreads, s, N, (const double*)psi, &dos->amax_psi);
  launch(p, k_sn_power_norm, gn, kThreads, s, n, G, (const int*)d.mat.as<int>(), (const double*)d.vol.as<double>(),
         (const double*)d.ksf.as<double>(), (const double*)phi0, dos, s1);
  launch(p, k_sn_power_fields, gn, kThreads, s, n, G, (const int*)d.mat.as<int>(), (const double*)d.vol.as<double>(),
         (const double*)d.ksf.as<double>(), (const double*)d.nsf.as<double>(), (const double*)phi0, opt->power,
         std::fmax(kZeroFlush, opt->tol_flux), d.phi.as<double>(), d.q.as<double>(), d.P.as<double>(), dos, s2);
  launch(p, k_sn_psi_norm, grid_for(N), kThreads, s, N, psi, opt->power, std::fmax(kZeroFlush, opt->tol_flux), dos,
         s1);
  PGPU_CUDA(cudaGetLastError());
  PGPU_CUDA(cudaEventRecord(e1, s));
  if ((st = read_outer(p, os))) return st;
  float ms = 0.f;
  PGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  stats->keff = os.k;
  stats->outer_iterations = std::min(outer, opt->max_outer);
  stats->inner_iterations = inner_total;
  stats->sweeps = d.sweeps;
  stats->residual = change;
  stats->seconds = ms * 1e-3;
  if (!converged) return fail(PGPU_ERR_NOT_CONVERGED, "SN power iteration reached max_outer without converging");
  if (os.negatives > 0) return fail(PGPU_ERR_NEGATIVE_FLUX, "negative values in the scalar- or angular-flux solution");
  return PGPU_OK;
}

}  // namespace

int sn_solve(pgpu_problem* p, const pgpu_options* opt, pgpu_stats* stats) {
  if (opt->precision == PGPU_MIXED) {
    int st = make_fp32(p);
    if (st) return st;
    if (!p->sn->psi32.ptr) {
      st = dev_alloc(p->sn->psi32, (size_t)p->sn->n * p->sn->G * p->sn->M * 4, &p->bytes, p->stream);
      if (st) return st;
    }
    return solve_T<float>(p, opt, stats);
  }
  return solve_T<double>(p, opt, stats);
}

int sn_get_flux(pgpu_problem* p, double* phi) {
  SNData& d = *p->sn;
  PGPU_CUDA(cudaMemcpyAsync(phi, d.phi.ptr, (size_t)d.n * d.G * 8, cudaMemcpyDeviceToHost, p->stream));
  PGPU_CUDA(cudaStreamSynchronize(p->stream));
  return PGPU_OK;
}

int sn_get_angular(pgpu_problem* p, double* psi) {
  SNData& d = *p->sn;
  PGPU_CUDA(cudaMemcpyAsync(psi, d.psi.ptr, (size_t)d.n * d.G * d.M * 8, cudaMemcpyDeviceToHost, p->stream));
  PGPU_CUDA(cudaStreamSynchronize(p->stream));
  return PGPU_OK;
}

int sn_get_power(pgpu_problem* p, double* q, double* P, double* total) {
  SNData& d = *p->sn;
  if (q) PGPU_CUDA(cudaMemcpyAsync(q, d.q.ptr, (size_t)d.n * 8, cudaMemcpyDeviceToHost, p->stream));
  if (P) PGPU_CUDA(cudaMemcpyAsync(P, d.P.ptr, (size_t)d.n * 8, cudaMemcpyDeviceToHost, p->stream));
  SNOuter os;
  if (int rst = read_small(&os, d.oscal.ptr, sizeof(os), p->stream)) return rst;
  if (total) *total = os.total_power;
  return PGPU_OK;
}

void sn_destroy(pgpu_problem* p) {
  delete p->sn;
  p->sn = nullptr;
}

// Plan of the column sweep of an extruded mesh (prisms stacked in layers, cells numbered
// layer by layer as the extruded-mesh reader does): every cell's lateral faces repeat the
// layer-0 cell's (same normals, neighbours in the same layer), z faces link consecutive
// layers.  A task is one column (all layers of a layer-0 cell) for one sweep pattern and
// one chunk of groups; it waits for the columns upwind of it across lateral faces (the
// columns' graph per pattern must be acyclic) and walks its layers in the pattern's z
// direction.  Returns false (level sweeps are used) when the mesh does not qualify.
struct ColPlan {
  int nxy = 0, nz = 0, nd = 0, gchunk = 1, nchunk = 1, ntasks = 0;
  std::vector<int> up;      // [npat][nxy][kColUp] lateral inflow face indices (-1: none)
  std::vector<int> zm, zp;  // [nxy] index of the -z / +z face (-1: none)
  std::vector<int> pat_sz;  // [npat] +1 / -1: the pattern's layer order (0: single layer)
  std::vector<int> order;   // [ntasks] (column * npat + pattern) * nchunk + chunk, by column level
};

static bool col_plan(const pgpu_sn_operator* op, const Schedule& S, ColPlan& C) {
  const int n = op->num_cells, F = op->num_faces;
  auto nrm = [&](int f, int i) { return op->normals + ((size_t)f * n + i) * 3; };
  auto is_z = [&](const double* v, double s) { return v[0] == 0.0 && v[1] == 0.0 && v[2] == s; };
  // layer size: the +z neighbour of cell 0 (a single layer when it has none)
  int nxy = n;
  for (int f = 0; f < op->num_cell_faces[0]; f++)
    if (is_z(nrm(f, 0), 1.0) && op->face_kind[(size_t)f * n] == PGPU_FACE_INTERIOR) nxy = op->neighbors[(size_t)f * n];
  if (nxy <= 0 || n % nxy) return false;
  const int nz = n / nxy;
  C.nxy = nxy;
  C.nz = nz;
  C.zm.assign(nxy, -1);
  C.zp.assign(nxy, -1);
  for (int c = 0; c < nxy; c++)
    for (int f = 0; f < op->num_cell_faces[c]; f++) {
      if (is_z(nrm(f, c), -1.0)) C.zm[c] = f;
      else if (is_z(nrm(f, c), 1.0)) C.zp[c] = f;
      else if (nrm(f, c)[2] != 0.0) return false;  // tilted face
    }
  // a single layer has no z order: its z faces must not carry reflective inflow
  if (nz == 1)
    for (int c = 0; c < nxy; c++)
      for (int f : {C.zm[c], C.zp[c]})
        if (f >= 0 && op->face_kind[(size_t)f * n + c] == PGPU_FACE_REFLECTIVE) return false;
  for (int k = 0; k < nz; k++)
    for (int c = 0; c < nxy; c++) {
      const int i = k * nxy + c;
      if (op->num_cell_faces[i] != op->num_cell_faces[c]) return false;
      for (int f = 0; f < op->num_cell_faces[c]; f++) {
        const size_t o = (size_t)f * n + i, o0 = (size_t)f * n + c;
        const double *a = nrm(f, i), *b = nrm(f, c);
        if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2]) return false;
        const int kd = op->face_kind[o], j = op->neighbors[o];
        if (f == C.zm[c] || f == C.zp[c]) {
          const int k2 = f == C.zm[c] ? k - 1 : k + 1;
          const bool inside = k2 >= 0 && k2 < nz;
          if (inside != (kd == PGPU_FACE_INTERIOR)) return false;
          if (inside && j != i + (k2 - k) * nxy) return false;
        } else {
          if (kd != op->face_kind[o0]) return false;
          if (kd == PGPU_FACE_INTERIOR && j != op->neighbors[o0] + k * nxy) return false;
        }
      }
    }
  // per pattern: layer order, lateral inflow faces of every column, column levels
  const int npat = S.npat;
  C.nd = 0;
  for (int p = 0; p < npat; p++) C.nd = std::max(C.nd, S.pat_dirs_ptr[p + 1] - S.pat_dirs_ptr[p]);
  if (C.nd > 32) return false;
  C.gchunk = std::max(1, std::min(op->num_groups, 32 / C.nd));
  C.nchunk = (op->num_groups + C.gchunk - 1) / C.gchunk;
  C.pat_sz.assign(npat, 0);
  C.up.assign((size_t)npat * nxy * kColUp, -1);
  std::vector<int> level((size_t)npat * nxy, 0);
  int maxlev = 0;
  for (int p = 0; p < npat; p++) {
    const int d0 = S.pat_dirs_ptr[p];
    const double* dir = op->directions + (size_t)S.pat_dirs[d0] * 3;
    if (nz > 1) {
      int sz = 0;
      for (int k = d0; k < S.pat_dirs_ptr[p + 1]; k++) {
        const double dz = op->directions[(size_t)S.pat_dirs[k] * 3 + 2];
        const int s = dz > 0.0 ? 1 : (dz < 0.0 ? -1 : 0);
        if (s == 0 || (sz != 0 && s != sz)) return false;
        sz = s;
      }
      C.pat_sz[p] = sz;
    }
    std::vector<int> indeg(nxy, 0), head(nxy + 1, 0), adj;
    for (int c = 0; c < nxy; c++) {
      int u = 0;
      for (int f = 0; f < op->num_cell_faces[c]; f++) {
        if (f == C.zm[c] || f == C.zp[c]) continue;
        const double* v = nrm(f, c);
        const int kd = op->face_kind[(size_t)f * n + c];
        if (!(kd == PGPU_FACE_INTERIOR || kd == PGPU_FACE_REFLECTIVE)) continue;
        // an interior face's sign is the pattern's; a reflective face's normal need not be
        // an interior normal, so it is an inflow face if any direction enters through it
        // (the per-direction coefficient is zero for the others)
        bool inflow = false;
        for (int k = d0; k < S.pat_dirs_ptr[p + 1] && !inflow; k++) {
          const double* dk = kd == PGPU_FACE_INTERIOR ? dir : op->directions + (size_t)S.pat_dirs[k] * 3;
          inflow = dk[0] * v[0] + dk[1] * v[1] + dk[2] * v[2] < 0.0;
        }
        if (!inflow) continue;
        if (u == kColUp) return false;
        C.up[((size_t)p * nxy + c) * kColUp + u++] = f;
        if (kd == PGPU_FACE_INTERIOR) {
          head[op->neighbors[(size_t)f * n + c] + 1]++;
          indeg[c]++;
        }
      }
    }
    for (int c = 0; c < nxy; c++) head[c + 1] += head[c];
    adj.assign(head[nxy], 0);
    std::vector<int> fill(head.begin(), head.end() - 1);
    for (int c = 0; c < nxy; c++)
      for (int u = 0; u < kColUp; u++) {
        const int f = C.up[((size_t)p * nxy + c) * kColUp + u];
        if (f >= 0 && op->face_kind[(size_t)f * n + c] == PGPU_FACE_INTERIOR) adj[fill[op->neighbors[(size_t)f * n + c]]++] = c;
      }
    std::vector<int> queue;
    queue.reserve(nxy);
    for (int c = 0; c < nxy; c++)
      if (indeg[c] == 0) queue.push_back(c);
    for (size_t q = 0; q < queue.size(); q++) {
      const int c = queue[q];
      for (int e = head[c]; e < head[c + 1]; e++) {
        const int c2 = adj[e];
        level[(size_t)p * nxy + c2] = std::max(level[(size_t)p * nxy + c2], level[(size_t)p * nxy + c] + 1);
        if (--indeg[c2] == 0) queue.push_back(c2);
      }
    }
    if ((int)queue.size() != nxy) return false;  // the columns' upwind graph has a cycle
    for (int c = 0; c < nxy; c++) maxlev = std::max(maxlev, level[(size_t)p * nxy + c]);
  }
  // tasks level by level (every pattern's columns of level L, all chunks): a task's
  // upwind tasks always come earlier
  std::vector<int> cnt(maxlev + 2, 0);
  for (int p = 0; p < npat; p++)
    for (int c = 0; c < nxy; c++) cnt[level[(size_t)p * nxy + c] + 1] += C.nchunk;
  for (int L = 0; L <= maxlev; L++) cnt[L + 1] += cnt[L];
  C.ntasks = cnt[maxlev + 1];
  C.order.assign(C.ntasks, 0);
  for (int p = 0; p < npat; p++)
    for (int c = 0; c < nxy; c++)
      for (int ch = 0; ch < C.nchunk; ch++) C.order[cnt[level[(size_t)p * nxy + c]]++] = (c * npat + p) * C.nchunk + ch;
  (void)F;
  return true;
}

// Plan of the tiled sweep: verifies that the operator is a full Cartesian box in the
// reference's cell and face order, with sides that are multiples of 4 and one sign per
// axis for every sweep pattern; returns false (level sweeps are used) otherwise.
struct KbaPlan {
  int t[3];  // tile shape
  int ntx, nty, ntz, nd, gchunk, nchunk, ntasks, npat;
  std::vector<int> tiles, pat_sign, pat_dirs_ptr, pat_dirs;
  std::vector<int> order;  // hand-out order of the tasks (empty: canonical)
};

// Directions per dataflow-sweep task at most (0: a whole octant).  Fewer directions per
// task make each task shorter, and the sweep's critical path is one task per tile
// diagonal; PGPU_FLOW_DIRS overrides it.
static int flow_dirs_max() {
  const char* e = std::getenv("PGPU_FLOW_DIRS");
  return e ? std::max(0, std::atoi(e)) : 0;
}

// Hand-out order of the dataflow sweep's tasks: PGPU_FLOW_STAGGER = "W:K" splits the
// independent pipelines (pattern, group chunk) into W waves and hands out wave w's tasks
// as if they were K*w tile diagonals later, so that the pipelines' fill and drain phases
// overlap instead of coinciding (unset: every pipeline starts at once).
static void flow_stagger(int& waves, int& offset) {
  waves = 1;
  offset = 0;
  const char* e = std::getenv("PGPU_FLOW_STAGGER");
  if (!e) return;
  int w = 1, k = 0;
  if (std::sscanf(e, "%d:%d", &w, &k) == 2 && w >= 1 && w <= 64 && k >= 0 && k <= 1024) {
    waves = w;
    offset = k;
  }
}

// Back-off between polls of an upwind tile's flag, in ns (PGPU_FLOW_SLEEP, default 32).
static int flow_sleep_ns() {
  const char* e = std::getenv("PGPU_FLOW_SLEEP");
  return e ? std::min(1000, std::max(0, std::atoi(e))) : 32;
}

// (group, direction) slots of one task at most: kFlowSlots, or PGPU_FLOW_SLOTS (1-64).
static int flow_slots() {
  const char* e = std::getenv("PGPU_FLOW_SLOTS");
  return e ? std::min(64, std::max(1, std::atoi(e))) : kFlowSlots;
}

static bool kba_plan(const pgpu_sn_operator* op, const Schedule& S, KbaPlan& K) {
  const int nx = op->cart_nx, ny = op->cart_ny, nz = op->cart_nz, n = op->num_cells;
  if (nx <= 0 || ny <= 0 || nz <= 0 || (long long)nx * ny * nz != n || op->num_faces != 6) return false;
  if (nx % 4 || ny % 4 || nz % 4) return false;
  // face f: normal and neighbour offset in the reference's order -y, +x, +y, -x, -z, +z
  const int nrm[6][3] = {{0, -1, 0}, {1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, 0, -1}, {0, 0, 1}};
  for (int z = 0, i = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++, i++) {
        if (op->num_cell_faces[i] != 6) return false;
        for (int f = 0; f < 6; f++) {
          const size_t o = (size_t)f * n + i;
          for (int a = 0; a < 3; a++)
            if (op->normals[o * 3 + a] != (double)nrm[f][a]) return false;
          const int x2 = x + nrm[f][0], y2 = y + nrm[f][1], z2 = z + nrm[f][2];
          const bool inside = x2 >= 0 && x2 < nx && y2 >= 0 && y2 < ny && z2 >= 0 && z2 < nz;
          if (inside != (op->face_kind[o] == PGPU_FACE_INTERIOR)) return false;
          if (inside && op->neighbors[o] != x2 + nx * (y2 + ny * z2)) return false;
        }
      }
  // the sweep's patterns: every octant's directions, in chunks of at most dmax
  const int dmax = flow_dirs_max();
  K.nd = 0;
  K.npat = 0;
  K.pat_dirs_ptr.assign(1, 0);
  K.pat_dirs.clear();
  for (int p = 0; p < S.npat; p++) {
    int sg[3] = {0, 0, 0};
    for (int k = S.pat_dirs_ptr[p]; k < S.pat_dirs_ptr[p + 1]; k++) {
      const double* d = op->directions + (size_t)S.pat_dirs[k] * 3;
      for (int a = 0; a < 3; a++) {
        const int s = d[a] > 0.0 ? 1 : (d[a] < 0.0 ? -1 : 0);
        if (s == 0 || (sg[a] != 0 && sg[a] != s)) return false;
        sg[a] = s;
      }
    }
    const int d0 = S.pat_dirs_ptr[p], ndp = S.pat_dirs_ptr[p + 1] - d0;
    const int parts = dmax > 0 ? (ndp + dmax - 1) / dmax : 1;
    for (int q = 0; q < parts; q++) {
      const int lo = d0 + (int)((long long)ndp * q / parts), hi = d0 + (int)((long long)ndp * (q + 1) / parts);
      for (int a = 0; a < 3; a++) K.pat_sign.push_back(sg[a]);
      for (int k = lo; k < hi; k++) K.pat_dirs.push_back(S.pat_dirs[k]);
      K.pat_dirs_ptr.push_back((int)K.pat_dirs.size());
      K.nd = std::max(K.nd, hi - lo);
      K.npat++;
    }
  }
  // groups per task: as many as fit in the task's (group, direction) slots
  K.gchunk = std::max(1, std::min(op->num_groups, flow_slots() / std::max(1, K.nd)));
  K.nchunk = (op->num_groups + K.gchunk - 1) / K.gchunk;
  // 8x8x4 tiles when the box divides into them, 4x4x4 otherwise
  const char* te = std::getenv("PGPU_FLOW_TILE");  // 4: force 4x4x4 tiles (measurement)
  const bool big = nx % 8 == 0 && ny % 8 == 0 && !(te && std::atoi(te) == 4);
  K.t[0] = big ? 8 : 4;
  K.t[1] = big ? 8 : 4;
  K.t[2] = 4;
  if (K.nd * K.gchunk > (big ? 256 : 128) || K.nd > kFlowMaxDirs) return false;
  K.ntx = nx / K.t[0];
  K.nty = ny / K.t[1];
  K.ntz = nz / K.t[2];
  // tiles in oriented coordinates, tile diagonal by tile diagonal
  const int ndiag = K.ntx + K.nty + K.ntz - 2;
  for (int D = 0; D < ndiag; D++)
    for (int tz = 0; tz < K.ntz; tz++)
      for (int ty = 0; ty < K.nty; ty++) {
        const int tx = D - ty - tz;
        if (tx < 0 || tx >= K.ntx) continue;
        K.tiles.push_back(tx);
        K.tiles.push_back(ty);
        K.tiles.push_back(tz);
      }
  const long long ntasks = (long long)K.ntx * K.nty * K.ntz * K.npat * K.nchunk;
  if (ntasks >= (1LL << 31)) return false;
  K.ntasks = (int)ntasks;
  int waves, offset;
  flow_stagger(waves, offset);
  K.order.clear();
  if (waves > 1 && offset > 0) {
    // keys: tile diagonal + wave offset; a stable sort keeps each pipeline's tasks in
    // diagonal order, so every task's upwind tasks are still handed out before it
    std::vector<std::pair<long long, int>> key(K.ntasks);
    for (int t = 0; t < K.ntasks; t++) {
      const int jp = t / K.nchunk, ch = t - jp * K.nchunk;
      const int j = jp / K.npat, pp = jp - j * K.npat;
      const int D = K.tiles[3 * j] + K.tiles[3 * j + 1] + K.tiles[3 * j + 2];
      const int q = pp * K.nchunk + ch;
      key[t] = {(long long)D + (long long)(q % waves) * offset, t};
    }
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<long long, int>& a, const std::pair<long long, int>& b) { return a.first < b.first; });
    K.order.resize(K.ntasks);
    for (int t = 0; t < K.ntasks; t++) K.order[t] = key[t].second;
  }
  return true;
}

// Cell classes of the sweeps' coefficient tables: cells with the same material, volume
// and, per face, kind, normal class and sweep weights (equal to 2^-36 relative) have the
// same coefficient rows for every group and direction.  Returns false when the table would hold more than
// kMaxClassTable bytes in FP64 (the per-row reciprocal diagonal is used instead).
constexpr size_t kMaxClassTable = 8u << 20;
// the level sweep's rows hold 1 + F values (the boundary layers of an unstructured lattice
// give a few hundred classes); its table may take 64 MiB in FP64, half of L2 in FP32
constexpr size_t kMaxLevelClassTable = 64u << 20;

static bool kba_classes(const pgpu_sn_operator* op, const std::vector<unsigned char>& ncls,
                        const std::vector<double>& wout, const std::vector<double>& windiag,
                        const std::vector<double>& win, std::vector<unsigned short>& ccls, std::vector<int>& rep,
                        int values_per_row = 4, size_t max_bytes = kMaxClassTable) {
  const int n = op->num_cells, F = op->num_faces, G = op->num_groups, M = op->num_dirs;
  const size_t per_class = (size_t)G * M * values_per_row * sizeof(double);
  std::map<std::vector<unsigned long long>, int> ids;
  std::vector<unsigned long long> key((size_t)2 + (size_t)F * 5), last;
  int last_id = -1;  // the previous cell's class: neighbouring cells mostly share one
  // values that differ only in their last 16 mantissa bits (relative 2^-36, e.g. cell
  // volumes of a lattice computed from rounded coordinates) share a class; the class
  // uses its first cell's exact values
  auto bits = [](double v) {
    unsigned long long u;
    std::memcpy(&u, &v, sizeof(u));
    return u & ~0xFFFFull;
  };
  ccls.assign(n, 0);
  rep.clear();
  for (int i = 0; i < n; i++) {
    key[0] = (unsigned long long)op->materials[i];
    key[1] = bits(op->volumes[i]);
    for (int f = 0; f < F; f++) {
      const size_t o = (size_t)f * n + i;
      unsigned long long* k = key.data() + 2 + (size_t)f * 5;
      k[0] = (unsigned long long)(unsigned)op->face_kind[o];
      k[1] = ncls[o];
      k[2] = bits(wout[o]);
      k[3] = bits(windiag[o]);
      k[4] = bits(win[o]);
    }
    int id;
    if (last_id >= 0 && key == last) {
      id = last_id;
    } else {
      auto it = ids.find(key);
      if (it == ids.end()) {
        id = (int)rep.size();
        if (id > 65535 || (size_t)(id + 1) * per_class > max_bytes) return false;
        ids.emplace(key, id);
        rep.push_back(i);
      } else {
        id = it->second;
      }
      last = key;
      last_id = id;
    }
    ccls[i] = (unsigned short)id;
  }
  return true;
}

// Cell order of the two tile shapes, diagonal by diagonal (local cell lx + TX*(ly + TY*lz)).
static void tile_order(int TX, int TY, int TZ, unsigned char* cells, int* dptr) {
  int k = 0;
  for (int dd = 0; dd < TX + TY + TZ - 2; dd++) {
    dptr[dd] = k;
    for (int lz = 0; lz < TZ; lz++)
      for (int ly = 0; ly < TY; ly++)
        for (int lx = 0; lx < TX; lx++)
          if (lx + ly + lz == dd) cells[k++] = (unsigned char)(lx + TX * (ly + TY * lz));
  }
  dptr[TX + TY + TZ - 2] = k;
}

static int kba_tables() {
  unsigned char c444[64], c884[256];
  int d444[11], d884[19];
  tile_order(4, 4, 4, c444, d444);
  tile_order(8, 8, 4, c884, d884);
  PGPU_CUDA(cudaMemcpyToSymbol(c_cell444, c444, sizeof(c444)));
  PGPU_CUDA(cudaMemcpyToSymbol(c_dptr444, d444, sizeof(d444)));
  PGPU_CUDA(cudaMemcpyToSymbol(c_cell884, c884, sizeof(c884)));
  PGPU_CUDA(cudaMemcpyToSymbol(c_dptr884, d884, sizeof(d884)));
  return PGPU_OK;
}

}  // namespace pgpu

extern "C" {

int pgpu_sn_create(int device, const pgpu_sn_operator* op, pgpu_problem** out) {
  using namespace pgpu;
  if (!op || !out) return fail(PGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  const int n = op->num_cells, G = op->num_groups, M = op->num_dirs, F = op->num_faces, nm = op->num_materials;
  if (n < 1 || G < 1 || M < 1 || F < 1 || nm < 1) return fail(PGPU_ERR_INVALID, "bad operator sizes");
  if ((long long)n * G * M >= (1LL << 40)) return fail(PGPU_ERR_INVALID, "operator too large");
  if (op->use_ls && !op->ls_weight) return fail(PGPU_ERR_INVALID, "use_ls set without ls_weight");
  for (int i = 0; i < n; i++) {
    if (op->materials[i] < 0 || op->materials[i] >= nm) return fail(PGPU_ERR_INVALID, "material index out of range");
    if (op->num_cell_faces[i] < 0 || op->num_cell_faces[i] > F) return fail(PGPU_ERR_INVALID, "bad face count");
  }
  bool upwind = true;
  std::vector<int> rslot((size_t)F * n, -1), slot_cell, slot_face;
  std::vector<double> lsdiag((size_t)F * n, 0.0);
  for (int i = 0; i < n; i++)
    for (int f = 0; f < op->num_cell_faces[i]; f++) {
      const size_t o = (size_t)f * n + i;
      const int k = op->face_kind[o];
      if (k == PGPU_FACE_INTERIOR) {
        if (op->neighbors[o] < 0 || op->neighbors[o] >= n) return fail(PGPU_ERR_INVALID, "neighbour index out of range");
        if (op->gauss[o * 4 + 1] != 0.0 || op->gauss[o * 4 + 2] != 0.0) upwind = false;
      } else if (k == PGPU_FACE_REFLECTIVE) {
        if (op->reflect_axis[o] < 0 || op->reflect_axis[o] > 2) return fail(PGPU_ERR_INVALID, "bad reflection axis");
        rslot[o] = (int)slot_cell.size();
        slot_cell.push_back(i);
        slot_face.push_back(f);
      } else if (k == PGPU_FACE_VACUUM) {
        if (op->use_ls)
          for (int f2 = 0; f2 < op->num_cell_faces[i]; f2++)
            if (op->face_kind[(size_t)f2 * n + i] == PGPU_FACE_INTERIOR) lsdiag[o] += op->ls_weight[o * F + f2];
      } else if (k != PGPU_FACE_NONE) {
        return fail(PGPU_ERR_INVALID, "bad face kind");
      }
    }
  for (int m = 0; m < M * 3; m++)
    if (op->reflected[m] < 0 || op->reflected[m] >= M) return fail(PGPU_ERR_INVALID, "bad reflected direction");
  if ((long long)n * G * M >= (1LL << 31)) return fail(PGPU_ERR_INVALID, "more than 2^31 angular unknowns");
  // sweep face weights and the table of mu over distinct face normals (SweepFaces)
  std::vector<double> wout((size_t)F * n, 0.0), windiag((size_t)F * n, 0.0), winw((size_t)F * n, 0.0);
  std::vector<unsigned char> cls((size_t)F * n, 0);
  NormalIds cls_of(F, 1e12);
  std::vector<const double*> cls_nrm;
  bool use_tab = true;
  for (int i = 0; i < n; i++)
    for (int f = 0; f < op->num_cell_faces[i]; f++) {
      const size_t o = (size_t)f * n + i;
      const double A = op->areas[o];
      const int k = op->face_kind[o];
      if (k == PGPU_FACE_INTERIOR) {
        wout[o] = op->gauss[o * 4 + 0] * A;
        windiag[o] = op->gauss[o * 4 + 2] * A;
        winw[o] = op->gauss[o * 4 + 3] * A;
      } else if (k == PGPU_FACE_VACUUM) {
        wout[o] = A * (1.0 - lsdiag[o]);
      } else if (k == PGPU_FACE_REFLECTIVE) {
        wout[o] = A;
        winw[o] = A;
      }
      const double* nr = op->normals + o * 3;
      const int id = cls_of.id(f, nr);
      if (id == (int)cls_nrm.size()) cls_nrm.push_back(nr);
      if (id > 255) use_tab = false;
      cls[o] = (unsigned char)(id & 255);
    }
  std::vector<double> mutab;
  if (use_tab) {
    mutab.assign(cls_nrm.size() * M, 0.0);
    for (size_t c = 0; c < cls_nrm.size(); c++)
      for (int m = 0; m < M; m++) {
        const double* d0 = op->directions + (size_t)m * 3;
        mutab[c * M + m] = d0[0] * cls_nrm[c][0] + d0[1] * cls_nrm[c][1] + d0[2] * cls_nrm[c][2];
      }
  }
  Schedule sched;
  int st = build_schedule(op, sched, false);
  if (st) return st;
  KbaPlan kp;
  const bool tiled = kba_plan(op, sched, kp);
  if (!tiled && (st = build_schedule(op, sched, true))) return st;
  PGPU_CUDA(cudaSetDevice(device));
  pgpu_problem* p = new pgpu_problem();
  p->kind = 2;
  p->device = device;
  p->num_cells = n;
  p->num_groups = G;
  p->num_dirs = M;
  p->sn = new SNData();
  SNData& d = *p->sn;
  d.n = n;
  d.G = G;
  d.M = M;
  d.F = F;
  d.nm = nm;
  d.use_ls = op->use_ls;
  d.upwind = upwind;
  d.nrefl = (int)slot_cell.size();
  d.sched = sched;
  st = PGPU_OK;
  auto up = [&](DevBuf& b, const void* h, size_t bytes) {
    if (st == PGPU_OK) st = dev_upload(b, h, bytes, &p->bytes, p->stream);
    p->uploaded += (long long)bytes;
  };
  auto al = [&](DevBuf& b, size_t bytes) {
    if (st == PGPU_OK) st = dev_alloc(b, bytes, &p->bytes, p->stream);
  };
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) st = fail(PGPU_ERR_CUDA, "stream");
  const size_t Fn = (size_t)F * n;
  up(d.nf, op->num_cell_faces, (size_t)n * 4);
  up(d.kind, op->face_kind, Fn * 4);
  up(d.nbr, op->neighbors, Fn * 4);
  up(d.raxis, op->reflect_axis, Fn * 4);
  up(d.rslot, rslot.data(), Fn * 4);
  up(d.mat, op->materials, (size_t)n * 4);
  up(d.refl, op->reflected, (size_t)M * 3 * 4);
  up(d.area, op->areas, Fn * 8);
  up(d.nrm, op->normals, Fn * 3 * 8);
  up(d.gauss, op->gauss, Fn * 4 * 8);
  if (op->use_ls) up(d.lsw, op->ls_weight, Fn * F * 8);
  up(d.lsdiag, lsdiag.data(), Fn * 8);
  up(d.vol, op->volumes, (size_t)n * 8);
  up(d.dirs, op->directions, (size_t)M * 3 * 8);
  up(d.w, op->weights, (size_t)M * 8);
  up(d.st, op->sigma_t, (size_t)nm * G * 8);
  up(d.ss, op->sigma_s, (size_t)nm * G * G * 8);
  up(d.chi, op->chi, (size_t)nm * G * 8);
  up(d.nsf, op->nu_sigma_f, (size_t)nm * G * 8);
  up(d.ksf, op->kappa_sigma_f, (size_t)nm * G * 8);
  up(d.d_pat_dirs_ptr, sched.pat_dirs_ptr.data(), sched.pat_dirs_ptr.size() * 4);
  up(d.d_pat_dirs, sched.pat_dirs.data(), sched.pat_dirs.size() * 4);
  up(d.d_pat_lev_ptr, sched.pat_lev_ptr.data(), sched.pat_lev_ptr.size() * 4);
  up(d.d_pat_nlev, sched.pat_nlev.data(), sched.pat_nlev.size() * 4);
  up(d.d_lev_ptr, sched.lev_ptr.data(), sched.lev_ptr.size() * 4);
  up(d.d_order, sched.order.data(), sched.order.size() * 4);
  d.use_tab = use_tab;
  up(d.cls, cls.data(), Fn);
  if (use_tab) up(d.mutab, mutab.data(), mutab.size() * 8);
  up(d.wout, wout.data(), Fn * 8);
  up(d.windiag, windiag.data(), Fn * 8);
  up(d.win, winw.data(), Fn * 8);
  if (st == PGPU_OK && tiled) {
    if ((st = kba_tables()) == PGPU_OK) {
      d.kba = true;
      d.kba_nx = op->cart_nx;
      d.kba_ny = op->cart_ny;
      d.kba_ntx = kp.ntx;
      d.kba_nty = kp.nty;
      d.kba_ntz = kp.ntz;
      d.kba_nd = kp.nd;
      d.kba_ntasks = kp.ntasks;
      d.kba_nchunk = kp.nchunk;
      d.kba_gchunk = kp.gchunk;
      d.kba_npat = kp.npat;
      for (int a = 0; a < 3; a++) d.kba_t[a] = kp.t[a];
      up(d.d_tiles, kp.tiles.data(), kp.tiles.size() * 4);
      if (!kp.order.empty()) up(d.d_task_order, kp.order.data(), kp.order.size() * 4);
      d.flow_sleep = flow_sleep_ns();
      // PGPU_FLOW_TRACE = "<sweep index>:<file>": record the timeline of that sweep of every
      // solve (measurement only)
      if (const char* te = std::getenv("PGPU_FLOW_TRACE")) {
        const char* colon = std::strchr(te, ':');
        if (colon && colon[1]) {
          d.trace_sweep = std::atoi(te);
          d.trace_file = colon + 1;
          al(d.trace_buf, (size_t)kp.ntasks * 5 * 8);
        }
      }
      up(d.d_pat_sign, kp.pat_sign.data(), kp.pat_sign.size() * 4);
      up(d.d_fpat_dirs_ptr, kp.pat_dirs_ptr.data(), kp.pat_dirs_ptr.size() * 4);
      up(d.d_fpat_dirs, kp.pat_dirs.data(), kp.pat_dirs.size() * 4);
      std::vector<unsigned short> ccls;
      std::vector<int> crep;
      if (kba_classes(op, cls, wout, windiag, winw, ccls, crep)) {
        d.ncls = (int)crep.size();
        up(d.d_ccls, ccls.data(), ccls.size() * 2);
        up(d.d_crep, crep.data(), crep.size() * 4);
        // per tile: its distinct classes (first kTileClasses) and each cell's index there
        const int ntl = kp.ntx * kp.nty * kp.ntz, nx = op->cart_nx, ny = op->cart_ny;
        std::vector<int> tcl((size_t)ntl * kTileClasses, -1), tnc(ntl, 0);
        std::vector<unsigned char> lcl(n, 0);
        for (int i = 0; i < n; i++) {
          const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
          const int tb = ((z / kp.t[2]) * kp.nty + y / kp.t[1]) * kp.ntx + x / kp.t[0];
          int* lst = tcl.data() + (size_t)tb * kTileClasses;
          int k = 0;
          while (k < std::min(tnc[tb], kTileClasses) && lst[k] != (int)ccls[i]) k++;
          if (k == std::min(tnc[tb], kTileClasses)) {
            if (tnc[tb] < kTileClasses) lst[k] = ccls[i];
            tnc[tb]++;
          }
          lcl[i] = (unsigned char)std::min(k, 255);
        }
        up(d.d_tile_cls, tcl.data(), tcl.size() * 4);
        up(d.d_tile_ncls, tnc.data(), tnc.size() * 4);
        up(d.d_cell_lcls, lcl.data(), lcl.size());
      }
      al(d.flow_sync, sizeof(FlowSync));
      al(d.flow_flags, (size_t)kp.ntasks * 4);
      if (st == PGPU_OK && (cudaMemsetAsync(d.flow_sync.ptr, 0, sizeof(FlowSync), p->stream) != cudaSuccess ||
                            cudaMemsetAsync(d.flow_flags.ptr, 0, (size_t)kp.ntasks * 4, p->stream) != cudaSuccess))
        st = fail(PGPU_ERR_CUDA, "clearing the sweep flags");
    }
  }
  if (st == PGPU_OK && !tiled && use_tab) {
    // level sets: per-class coefficient rows [rd, a_f] instead of a reciprocal diagonal per
    // (cell, group, direction), when the classes' table stays small
    std::vector<unsigned short> ccls;
    std::vector<int> crep;
    if (kba_classes(op, cls, wout, windiag, winw, ccls, crep, 1 + F, kMaxLevelClassTable)) {
      d.ncls = (int)crep.size();
      up(d.d_ccls, ccls.data(), ccls.size() * 2);
      up(d.d_crep, crep.data(), crep.size() * 4);
      // extruded meshes (and boxes the tiles do not fit): the column sweep instead of one
      // launch per level (PGPU_SWEEP_COLUMNS=0 keeps the level sets, for measurement)
      ColPlan cp;
      const char* ce = std::getenv("PGPU_SWEEP_COLUMNS");
      if (!(ce && std::atoi(ce) == 0) && col_plan(op, sched, cp)) {
        d.col = true;
        d.col_nxy = cp.nxy;
        d.col_nz = cp.nz;
        d.col_nd = cp.nd;
        d.col_ntasks = cp.ntasks;
        d.col_gchunk = cp.gchunk;
        d.col_nchunk = cp.nchunk;
        d.flow_sleep = flow_sleep_ns();
        up(d.d_col_up, cp.up.data(), cp.up.size() * 4);
        up(d.d_col_zm, cp.zm.data(), cp.zm.size() * 4);
        up(d.d_col_zp, cp.zp.data(), cp.zp.size() * 4);
        up(d.d_col_sz, cp.pat_sz.data(), cp.pat_sz.size() * 4);
        up(d.d_col_order, cp.order.data(), cp.order.size() * 4);
        const size_t nflags = (size_t)sched.npat * cp.nchunk * cp.nxy;  // 64-bit progress words
        al(d.flow_sync, sizeof(FlowSync));
        al(d.flow_flags, nflags * 8);
        if (st == PGPU_OK && (cudaMemsetAsync(d.flow_sync.ptr, 0, sizeof(FlowSync), p->stream) != cudaSuccess ||
                              cudaMemsetAsync(d.flow_flags.ptr, 0, nflags * 8, p->stream) != cudaSuccess))
          st = fail(PGPU_ERR_CUDA, "clearing the sweep flags");
      }
    }
  }
  if (d.nrefl) {
    up(d.d_slot_cell, slot_cell.data(), slot_cell.size() * 4);
    up(d.d_slot_face, slot_face.data(), slot_face.size() * 4);
  }
  {
    // incoming-direction lists of the reflective slots, one per distinct face normal
    // (all directions when mu comes from the normals rather than the table)
    std::map<int, int> list_of;
    std::vector<int> rkind(std::max<size_t>(1, slot_cell.size()), 0);
    std::vector<std::vector<int>> lists;
    for (size_t s = 0; s < slot_cell.size(); s++) {
      const int c = use_tab ? cls[(size_t)slot_face[s] * n + slot_cell[s]] : -1;
      auto it = list_of.find(c);
      if (it == list_of.end()) {
        std::vector<int> lst;
        for (int m = 0; m < M; m++)
          if (c < 0 || !(mutab[(size_t)c * M + m] > 0.0)) lst.push_back(m);
        it = list_of.emplace(c, (int)lists.size()).first;
        lists.push_back(lst);
      }
      rkind[s] = it->second;
    }
    if (lists.empty()) lists.push_back({});
    int Mh = 1;
    for (auto& l : lists) Mh = std::max<int>(Mh, (int)l.size());
    std::vector<int> kmap(lists.size() * M, -1), klist(lists.size() * Mh, -1);
    for (size_t r = 0; r < lists.size(); r++)
      for (size_t k = 0; k < lists[r].size(); k++) {
        kmap[r * M + lists[r][k]] = (int)k;
        klist[r * Mh + k] = lists[r][k];
      }
    d.Mh = Mh;
    up(d.d_rkind, rkind.data(), rkind.size() * 4);
    up(d.d_kmap, kmap.data(), kmap.size() * 4);
    up(d.d_klist, klist.data(), klist.size() * 4);
  }
  const size_t nG = (size_t)n * G;
  al(d.psi, nG * M * 8);
  al(d.phi0, nG * 8);
  al(d.phi, nG * 8);
  al(d.src, nG * 8);
  al(d.fs, (size_t)n * 8);
  al(d.fs_old, (size_t)n * 8);
  al(d.q, std::max(nG, (size_t)n) * 8);
  al(d.P, (size_t)n * 8);
  al(d.oscal, sizeof(SNOuter));
  if (st == PGPU_OK && cudaStreamSynchronize(p->stream) != cudaSuccess) st = fail(PGPU_ERR_CUDA, "upload");
  if (st != PGPU_OK) {
    std::string msg = pgpu_last_error();
    pgpu_problem_destroy(p);
    return fail(st, msg);
  }
  *out = p;
  return PGPU_OK;
}

int pgpu_sn_apply(pgpu_problem* p, const double* x, double* y) {
  using namespace pgpu;
  if (!p || p->kind != 2) return fail(PGPU_ERR_INVALID, "not an SN problem");
  PGPU_CUDA(cudaSetDevice(p->device));
  SNData& d = *p->sn;
  const size_t N = (size_t)d.n * d.G * d.M;
  DevBuf xb, yb;
  int st;
  if ((st = dev_alloc(xb, N * 8, nullptr)) || (st = dev_alloc(yb, N * 8, nullptr))) return st;
  PGPU_CUDA(cudaMemcpyAsync(xb.ptr, x, N * 8, cudaMemcpyHostToDevice, p->stream));
  if ((st = apply_R<double>(p, make_op<double>(d), xb.as<double>(), yb.as<double>(), d.phi0.as<double>()))) return st;
  PGPU_CUDA(cudaMemcpyAsync(y, yb.ptr, N * 8, cudaMemcpyDeviceToHost, p->stream));
  PGPU_CUDA(cudaStreamSynchronize(p->stream));
  return PGPU_OK;
}

}  // extern "C"
