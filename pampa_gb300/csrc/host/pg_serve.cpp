// Serving: continuous batching of independent k-eigenvalue solves on one GPU.
//
// Requests (a diffusion or SN operator plus solve options) are copied at submission and
// queued in arrival order.  `slots` worker threads, each with its own problem and CUDA
// stream, take requests from the queue as soon as a slot is free and the request's device
// footprint fits in the server's share of HBM; the operator is uploaded, solved and freed
// by the worker, so operators and flux iterates stay resident only while their solve
// runs, and the kernels of concurrent solves overlap on the device.  Every solve uses the
// same deterministic kernels and its own device state, so a result does not depend on
// what else runs beside it.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "pampa_gb300.h"

namespace pgpu {
void set_error(const std::string& msg);  // the calling thread's pgpu_last_error()
}

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename T>
void own(std::vector<T>& dst, const T* src, size_t count) {
  if (src) dst.assign(src, src + count);
  else dst.clear();
}

template <typename T>
const T* ptr(const std::vector<T>& v) {
  return v.empty() ? nullptr : v.data();
}

// Deep copy of a diffusion operator.
struct OwnedDiffusion {
  pgpu_diffusion_operator op{};
  std::vector<int> nbr, mat;
  std::vector<double> off, diag, vol, ss, chi, nsf, ksf;
  explicit OwnedDiffusion(const pgpu_diffusion_operator& s) {
    const size_t n = (size_t)s.num_cells, G = (size_t)s.num_groups, F = (size_t)s.num_faces,
                 nm = (size_t)s.num_materials;
    own(nbr, s.neighbors, F * n);
    own(off, s.offdiag, F * n * G);
    own(diag, s.diag, n * G);
    own(mat, s.materials, n);
    own(vol, s.volumes, n);
    own(ss, s.sigma_s, nm * G * G);
    own(chi, s.chi, nm * G);
    own(nsf, s.nu_sigma_f, nm * G);
    own(ksf, s.kappa_sigma_f, nm * G);
    op = s;
    op.neighbors = ptr(nbr);
    op.offdiag = ptr(off);
    op.diag = ptr(diag);
    op.materials = ptr(mat);
    op.volumes = ptr(vol);
    op.sigma_s = ptr(ss);
    op.chi = ptr(chi);
    op.nu_sigma_f = ptr(nsf);
    op.kappa_sigma_f = ptr(ksf);
  }
};

// Deep copy of an SN operator.
struct OwnedSN {
  pgpu_sn_operator op{};
  std::vector<int> nf, kind, nbr, raxis, refl, mat;
  std::vector<double> area, nrm, gauss, lsw, vol, dirs, w, st, ss, chi, nsf, ksf;
  explicit OwnedSN(const pgpu_sn_operator& s) {
    const size_t n = (size_t)s.num_cells, G = (size_t)s.num_groups, F = (size_t)s.num_faces,
                 M = (size_t)s.num_dirs, nm = (size_t)s.num_materials;
    own(nf, s.num_cell_faces, n);
    own(kind, s.face_kind, F * n);
    own(nbr, s.neighbors, F * n);
    own(area, s.areas, F * n);
    own(nrm, s.normals, F * n * 3);
    own(gauss, s.gauss, F * n * 4);
    own(raxis, s.reflect_axis, F * n);
    own(lsw, s.use_ls ? s.ls_weight : nullptr, F * n * F);
    own(vol, s.volumes, n);
    own(dirs, s.directions, M * 3);
    own(w, s.weights, M);
    own(refl, s.reflected, M * 3);
    own(mat, s.materials, n);
    own(st, s.sigma_t, nm * G);
    own(ss, s.sigma_s, nm * G * G);
    own(chi, s.chi, nm * G);
    own(nsf, s.nu_sigma_f, nm * G);
    own(ksf, s.kappa_sigma_f, nm * G);
    op = s;
    op.num_cell_faces = ptr(nf);
    op.face_kind = ptr(kind);
    op.neighbors = ptr(nbr);
    op.areas = ptr(area);
    op.normals = ptr(nrm);
    op.gauss = ptr(gauss);
    op.reflect_axis = ptr(raxis);
    op.ls_weight = ptr(lsw);
    op.volumes = ptr(vol);
    op.directions = ptr(dirs);
    op.weights = ptr(w);
    op.reflected = ptr(refl);
    op.materials = ptr(mat);
    op.sigma_t = ptr(st);
    op.sigma_s = ptr(ss);
    op.chi = ptr(chi);
    op.nu_sigma_f = ptr(nsf);
    op.kappa_sigma_f = ptr(ksf);
  }
};

struct Request {
  long long id = 0;
  std::unique_ptr<OwnedDiffusion> diff;
  std::unique_ptr<OwnedSN> sn;
  pgpu_options opt{};
  int want_flux = 0;
  size_t bytes = 0;  // device footprint estimate used for admission
  // results
  bool done = false;
  int status = PGPU_OK;
  std::string error;
  pgpu_stats stats{};
  double keff = 0.0;
  std::vector<double> phi;
  double t_submit = 0.0, t_start = 0.0, t_done = 0.0;
};

}  // namespace

// device shares of all slots add up to this many devices (measured on the 256-request
// diffusion stream at 16 slots: 3 gave 50.2 solves/s and p99 468 ms, 2 gave 47.3 and 482)
constexpr int kShareOverlap = 3;

struct pgpu_server {
  int device = 0;
  int sm_share = 0;   // SMs each solve sizes its grids for (0: whole device)
  size_t budget = 0;  // bytes of HBM the in-flight solves may hold
  size_t held = 0;
  int running = 0;
  bool stop = false;
  long long next_id = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending;
  std::unordered_map<long long, std::unique_ptr<Request>> requests;
  std::vector<std::thread> workers;
};

namespace {

void run_request(pgpu_server* s, Request* r, int sm_share) {
  pgpu_problem* p = nullptr;
  int st = r->diff ? pgpu_diffusion_create(s->device, &r->diff->op, &p) : pgpu_sn_create(s->device, &r->sn->op, &p);
  if (st == PGPU_OK) st = pgpu_problem_set_sm_share(p, sm_share);
  if (st == PGPU_OK) st = pgpu_problem_solve(p, &r->opt, &r->stats);
  if (st == PGPU_OK) st = pgpu_problem_get_keff(p, &r->keff);
  if (st == PGPU_OK && r->want_flux) {
    const size_t nG = r->diff ? (size_t)r->diff->op.num_cells * r->diff->op.num_groups
                              : (size_t)r->sn->op.num_cells * r->sn->op.num_groups;
    r->phi.resize(nG);
    st = pgpu_problem_get_scalar_flux(p, r->phi.data());
  }
  if (st != PGPU_OK) r->error = pgpu_last_error();
  if (p) pgpu_problem_destroy(p);
  r->status = st;
  // the operator copy is no longer needed
  r->diff.reset();
  r->sn.reset();
}

void worker_loop(pgpu_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    Request* r = nullptr;
    int share = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // first in, first admitted: the head waits until its footprint fits beside the
      // solves in flight (it always fits an idle server: oversize requests are rejected
      // at submission)
      s->cv_work.wait(lk, [&] {
        return (s->stop && s->pending.empty()) ||
               (!s->pending.empty() && s->held + s->pending.front()->bytes <= s->budget);
      });
      if (s->pending.empty()) return;  // stopping and nothing left
      r = s->pending.front();
      s->pending.pop_front();
      s->held += r->bytes;
      s->running++;
      r->t_start = now_s();
      share = s->sm_share;
    }
    run_request(s, r, share);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->held -= r->bytes;
      s->running--;
      r->t_done = now_s();
      r->done = true;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
}

// Device bytes of a solve: operator arrays, FP32 copies for mixed precision and the
// solver's work vectors, with 25 % margin for allocator rounding and reduction buffers.
size_t estimate_diffusion(const pgpu_diffusion_operator& op, int precision) {
  const double n = op.num_cells, nG = n * op.num_groups, F = op.num_faces;
  double b = F * n * 4 + n * 4 + F * nG * 8 + nG * 8 + n * 8 + 14 * nG * 8 + 4 * n * 8;
  if (precision == PGPU_MIXED) b += (F + 1) * nG * 4 + n * 4 + 9 * nG * 4;
  return (size_t)(1.25 * b) + (8u << 20);
}

size_t estimate_sn(const pgpu_sn_operator& op, int precision) {
  const double n = op.num_cells, G = op.num_groups, M = op.num_dirs, F = op.num_faces;
  const double N = n * G * M, nG = n * G;
  // scalar-flux-space Krylov vectors for pure upwind faces without the LS correction,
  // angular-space vectors otherwise
  bool upwind = !op.use_ls;
  for (size_t o = 0; upwind && o < (size_t)op.num_faces * op.num_cells; o++)
    if (op.face_kind[o] == PGPU_FACE_INTERIOR && (op.gauss[o * 4 + 1] != 0.0 || op.gauss[o * 4 + 2] != 0.0))
      upwind = false;
  double nrefl = 0;
  for (size_t o = 0; o < (size_t)op.num_faces * op.num_cells; o++) nrefl += op.face_kind[o] == PGPU_FACE_REFLECTIVE;
  const double len = upwind ? nG + nrefl * G * M : N;
  const double es = precision == PGPU_MIXED ? 4.0 : 8.0;
  double b = F * n * 113.0 + n * 44.0 + (M < 64 ? M : 64) * n * 4.0  // operator, weights, schedule
             + 2.0 * N * 8.0 + 24.0 * nG * 8.0                      // psi, reciprocal diagonal, cell vectors
             + 35.0 * len * es + 3.0 * len * 8.0;                    // Krylov basis and FP64 state
  if (op.use_ls) b += F * F * n * 8.0;
  if (precision == PGPU_MIXED) b += F * n * 56.0 + 2.0 * N * 4.0;
  return (size_t)(1.25 * b) + (16u << 20);
}

int submit(pgpu_server* s, Request* r, long long* id) {
  if (r->bytes > s->budget) {
    delete r;
    return PGPU_ERR_NO_MEMORY;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    r->t_submit = now_s();
    s->requests.emplace(r->id, std::unique_ptr<Request>(r));
    s->pending.push_back(r);
    *id = r->id;
  }
  s->cv_work.notify_all();
  return PGPU_OK;
}

}  // namespace

extern "C" {

int pgpu_serve_create(int device, int slots, double hbm_fraction, pgpu_server** out) {
  if (!out || slots < 1 || slots > 256 || !(hbm_fraction > 0.0) || hbm_fraction > 1.0) return PGPU_ERR_INVALID;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return PGPU_ERR_CUDA;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return PGPU_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PGPU_ERR_CUDA;
  pgpu_server* s = new pgpu_server();
  s->device = device;
  s->budget = (size_t)(hbm_fraction * (double)free_b);
  // each solve gets kShareOverlap / slots of the device: the slots' small kernels run side
  // by side, and a large solve still reaches full bandwidth while the others are small
  s->sm_share = slots == 1 ? 0 : std::min(sms, (kShareOverlap * sms + slots - 1) / slots);
  for (int k = 0; k < slots; k++) s->workers.emplace_back(worker_loop, s);
  *out = s;
  return PGPU_OK;
}

long long pgpu_serve_budget_bytes(pgpu_server* s) { return s ? (long long)s->budget : 0; }

int pgpu_serve_set_sm_share(pgpu_server* s, int sms) {
  if (!s || sms < 0) return PGPU_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->sm_share = sms;
  return PGPU_OK;
}

int pgpu_serve_submit_diffusion(pgpu_server* s, const pgpu_diffusion_operator* op, const pgpu_options* opt,
                                int want_flux, long long* id) {
  if (!s || !op || !id) return PGPU_ERR_INVALID;
  Request* r = new Request();
  r->diff.reset(new OwnedDiffusion(*op));
  if (opt) r->opt = *opt;
  else pgpu_default_options(&r->opt);
  r->want_flux = want_flux;
  r->bytes = estimate_diffusion(*op, r->opt.precision);
  return submit(s, r, id);
}

int pgpu_serve_submit_sn(pgpu_server* s, const pgpu_sn_operator* op, const pgpu_options* opt, int want_flux,
                         long long* id) {
  if (!s || !op || !id) return PGPU_ERR_INVALID;
  Request* r = new Request();
  r->sn.reset(new OwnedSN(*op));
  if (opt) r->opt = *opt;
  else pgpu_default_options(&r->opt);
  r->want_flux = want_flux;
  r->bytes = estimate_sn(*op, r->opt.precision);
  return submit(s, r, id);
}

int pgpu_serve_poll(pgpu_server* s, long long id, int* done) {
  if (!s || !done) return PGPU_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->requests.find(id);
  if (it == s->requests.end()) return PGPU_ERR_INVALID;
  *done = it->second->done ? 1 : 0;
  return PGPU_OK;
}

int pgpu_serve_wait(pgpu_server* s, long long id, pgpu_stats* stats, double* keff, double* phi, double* times) {
  if (!s) return PGPU_ERR_INVALID;
  std::unique_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return PGPU_ERR_INVALID;
    Request* rp = it->second.get();
    s->cv_done.wait(lk, [&] { return rp->done; });
    r = std::move(it->second);
    s->requests.erase(it);
  }
  if (r->status != PGPU_OK) pgpu::set_error("request " + std::to_string(id) + ": " + r->error);
  if (stats) *stats = r->stats;
  if (keff) *keff = r->keff;
  if (phi && !r->phi.empty()) std::memcpy(phi, r->phi.data(), r->phi.size() * sizeof(double));
  if (times) {
    times[0] = r->t_start - r->t_submit;  // queueing
    times[1] = r->t_done - r->t_start;    // upload + solve + read-back
    times[2] = r->t_done - r->t_submit;   // latency
  }
  return r->status;
}

int pgpu_serve_destroy(pgpu_server* s) {
  if (!s) return PGPU_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
  return PGPU_OK;
}

}  // extern "C"
