// Solver classes behind the drop-in API: the Solver / NeutronicSolver interface
// (Solver.hxx:31-98, NeutronicSolver.hxx:6-75) and the host half of DiffusionSolver and
// SNSolver.  The host half reads the solver block, turns mesh + materials into the GPU
// operator layouts of pampa_gb300.h, and hands the solve to pgpu_*; nothing here
// iterates on the flux.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <climits>
#include <cmath>
#include <cstring>
#include <iomanip>
#include <iostream>

#include "pg_host.hpp"

namespace pg {

// ----------------------------------------------------------------------------------
// Solver: fields by name (Solver.cxx:18-43).
// ----------------------------------------------------------------------------------

int Solver::getField(double* v, const std::string& name) const {
  for (const auto& f : fields_)
    if (f.name == name) {
      if (!f.vec) return f.get(v);
      std::memcpy(v, f.vec->data(), f.vec->size() * sizeof(double));
      return 0;
    }
  PG_CHECK(true, "unable to find field '" + name + "'");
}

int Solver::setField(const double* v, const std::string& name) {
  for (auto& f : fields_)
    if (f.name == name) {
      if (!f.vec) return f.set(v);
      std::memcpy(f.vec->data(), v, f.vec->size() * sizeof(double));
      return 0;
    }
  PG_CHECK(true, "unable to find field '" + name + "'");
}

int Solver::fieldSize(const std::string& name, int& size) const {
  for (const auto& f : fields_)
    if (f.name == name) {
      size = (int)(f.vec ? f.vec->size() : f.size);
      return 0;
    }
  PG_CHECK(true, "unable to find field '" + name + "'");
}

// ----------------------------------------------------------------------------------
// NeutronicSolver
// ----------------------------------------------------------------------------------

NeutronicSolver::~NeutronicSolver() {
  if (problem_) pgpu_problem_destroy(problem_);
}

// Keys shared by DiffusionSolver::read and SNSolver::read (DiffusionSolver.cxx:4-85).
int NeutronicSolver::readCommon(const std::vector<std::string>& line, Tokens& tok,
                                const Mesh& mesh, bool& used) {
  used = true;
  const std::string& k = line[0];
  if (k == "energy-groups") {
    PG_CHECK(line.size() != 2, "wrong number of arguments for keyword '" + k + "'");
    PG_TRY(to_int(line[1], 1, INT_MAX, G_), "wrong number of energy groups");
  } else if (k == "bc") {
    PG_CHECK(line.size() < 3, "wrong number of arguments for keyword '" + k + "'");
    int ibc = -1;
    for (size_t b = 0; b < mesh.boundaries.size(); b++)
      if (mesh.boundaries[b] == line[1]) ibc = (int)b;
    PG_CHECK(ibc < 0, "wrong boundary name");
    has_bcs_ = true;
    PG_TRY(read_bc(line, 2, tok, bcs_[ibc + 1]), "wrong boundary condition");
  } else if (k == "power") {
    PG_CHECK(line.size() != 2, "wrong number of arguments for keyword '" + k + "'");
    PG_TRY(to_double(line[1], 0.0, DBL_MAX, power_), "wrong power level");
  } else if (k == "convergence") {
    // convergence errors of the output fields drive an implicit coupling (CouplingSolver)
    PG_CHECK(line.size() != 5, "wrong number of arguments for keyword '" + k + "'");
    if (line[1] == "power") {
      PG_TRY(read_convergence(line, 1, dq_), "wrong convergence error");
    } else if (line[1] == "production-rate") {
      PG_TRY(read_convergence(line, 1, dP_), "wrong convergence error");
    } else {
      PG_CHECK(true, "wrong field");
    }
  } else {
    used = false;
  }
  return 0;
}

const std::map<int, BoundaryCondition>& NeutronicSolver::boundaryConditions() const {
  // DiffusionSolver.cxx:91, SNSolver.cxx:346: the solver's own BCs replace the mesh's.
  return has_bcs_ ? bcs_ : mesh_->bcs;
}

int NeutronicSolver::initialize(const Mesh& mesh, const std::vector<Material>& mats,
                                const RunOptions& opt, bool transient) {
  mesh_ = &mesh;
  mats_ = &mats;
  opt_ = opt;
  opt_.gpu.power = power_;
  transient_ = transient;
  n0_ = -1;
  PG_CHECK(G_ < 1, "missing number of energy groups");
  for (const auto& m : mats)
    PG_TRY(m.check_for_solver(G_, name_ == "diffusion", transient), "wrong material data");
  const int n = mesh.num_cells;
  T_.assign(n, 0.0);
  S_.assign(n, 0.0);
  phi_.assign((size_t)n * G_, 0.0);
  q_.assign(n, 0.0);
  P_.assign(n, 0.0);
  fields_.clear();
  fields_.push_back({"temperature", &T_, true, false, nullptr});
  fields_.push_back({"delayed-source", &S_, true, false, nullptr});
  fields_.push_back({"scalar-flux", &phi_, false, false, nullptr});
  fields_.push_back({"power", &q_, false, true, dq_});
  fields_.push_back({"production-rate", &P_, false, true, dP_});
  return 0;
}

// NeutronicSolver::solve (NeutronicSolver.cxx:4-43): n = 0 is the k-eigenvalue solve,
// n > 0 a transient step.
int NeutronicSolver::solve(int n, double dt, double t) {
  if (n > 0) return solveTransient(n, dt, t);
  if (problem_ && temperatureChanged()) {  // feedback data: the operator follows the temperatures
    pgpu_problem_destroy(problem_);
    problem_ = nullptr;
  }
  if (!problem_) {
    buildCellMaterials();
    PG_TRY(buildProblem(), "unable to build the coefficient matrices");
  }
  int st = pgpu_problem_solve(problem_, &opt_.gpu, &stats_);
  PG_CHECK(st != PGPU_OK, std::string("GPU k-eigenvalue solve failed: ") + pgpu_last_error());
  PG_TRY(pgpu_problem_get_keff(problem_, &keff_), "unable to get keff");
  PG_TRY(pgpu_problem_get_scalar_flux(problem_, phi_.data()), "unable to get the scalar flux");
  PG_TRY(pgpu_problem_get_power(problem_, q_.data(), P_.data(), &total_power_),
         "unable to get the power");
  // calculatePowerAndProductionRate also sets the delayed source S = beta * P
  // (NeutronicSolver.cxx:81-116).
  for (int i = 0; i < mesh_->num_cells; i++) S_[i] = (*mats_)[mesh_->materials[i]].beta_total * P_[i];
  PG_TRY(fetchSolution(), "unable to get the solution");
  return 0;
}

// The constant data every cell sees: its material at the cell's temperature (the
// `temperature` field) when the material has feedback data, else the material itself;
// cell_mats_ holds each distinct (material, temperature) once and cell_mat_ indexes it.
void NeutronicSolver::buildCellMaterials() {
  const Mesh& mesh = *mesh_;
  cell_mats_.clear();
  cell_mat_.assign(mesh.num_cells, 0);
  feedback_ = false;
  for (const auto& m : *mats_) feedback_ |= m.feedback();
  if (!feedback_) {
    cell_mats_ = *mats_;
    cell_mat_ = mesh.materials;
    return;
  }
  std::map<std::pair<int, double>, int> index;
  for (int i = 0; i < mesh.num_cells; i++) {
    const int m = mesh.materials[i];
    const double t = (*mats_)[m].feedback() ? T_[i] : 0.0;
    auto it = index.find({m, t});
    if (it == index.end()) {
      Material md;
      (*mats_)[m].at(t, md);
      cell_mats_.push_back(md);
      it = index.emplace(std::make_pair(m, t), (int)cell_mats_.size() - 1).first;
    }
    cell_mat_[i] = it->second;
  }
  T_built_ = T_;
}

bool NeutronicSolver::temperatureChanged() const {
  if (!feedback_) return false;
  return T_ != T_built_;
}

// Time steps of solvers without one here.  For SN the reference assembles the step's
// angular-flux system (SNSolver.cxx:371-441) but solves it into the scalar-flux vector,
// whose size does not match (SNSolver.cxx:658-666), so its own step always stops with an
// error; this build reports the same failure, with the reason.
int NeutronicSolver::solveTransient(int n, double dt, double t) {
  (void)n;
  (void)dt;
  (void)t;
  PG_CHECK(name_ == "sn",
           "unable to solve the linear system (the SN time step solves an angular-flux system into the "
           "scalar-flux vector in the reference, whose sizes do not match)");
  PG_CHECK(true, "transient steps (n > 0) are not available for the " + name_ + " solver in this build");
}

// NeutronicSolver::calculatePowerAndProductionRate (NeutronicSolver.cxx:81-116) for a
// flux that is not normalised (transient steps): q_i = sum_g phi kappa_sigma_f V,
// P_i = sum_g phi nu_sigma_f V / keff, S_i = beta P_i, and the total power.
void NeutronicSolver::powerAndProduction() {
  const int n = mesh_->num_cells;
  total_power_ = 0.0;
  for (int i = 0; i < n; i++) {
    const Material& mat = cell_mats_[cell_mat_[i]];
    const double V = mesh_->volumes[i];
    q_[i] = 0.0;
    P_[i] = 0.0;
    for (int g = 0; g < G_; g++) {
      const double ph = phi_[(size_t)i * G_ + g];
      q_[i] += ph * mat.kappa_sigma_f[g] * V;
      P_[i] += ph * mat.nu_sigma_f[g] * V / keff_;
    }
    S_[i] = mat.beta_total * P_[i];
    total_power_ += q_[i];
  }
}

// NeutronicSolver::printLog (NeutronicSolver.cxx:119-127) through PhysicsSolver::output.
int NeutronicSolver::output(int n, bool write_mesh) const {
  if (!opt_.silent) {
    if (n == 0)
      std::cout << std::fixed << std::setprecision(6) << "Effective multiplication factor: " << keff_
                << "." << std::endl;
    std::cout << std::scientific << std::setprecision(3) << "Power: " << total_power_ << "."
              << std::endl;
  }
  if (write_mesh) PG_TRY(write_vtk_mesh("./output", n, opt_, *mesh_), "unable to write the mesh in .vtk format");
  PG_TRY(writeFields(n), "unable to write the solution");
  return 0;
}

// DiffusionSolver::writeVTK and writePETSc (DiffusionSolver.cxx:410-432).
int NeutronicSolver::writeFields(int n) const {
  const int nc = mesh_->num_cells;
  PG_TRY(write_vtk_field("./output", n, opt_, "flux", phi_, nc, G_), "unable to write the scalar flux");
  PG_TRY(write_vtk_field("./output", n, opt_, "power", q_, nc), "unable to write the thermal power");
  PG_TRY(write_petsc_vec("scalar_flux", n, opt_, phi_), "unable to write the scalar flux");
  return 0;
}

int NeutronicSolver::problem(pgpu_problem** out) {
  if (!problem_) {
    buildCellMaterials();
    PG_TRY(buildProblem(), "unable to build the coefficient matrices");
  }
  *out = problem_;
  return 0;
}

int NeutronicSolver::finalize() {
  if (problem_) pgpu_problem_destroy(problem_);
  problem_ = nullptr;
  return 0;
}

// ----------------------------------------------------------------------------------
// Diffusion
// ----------------------------------------------------------------------------------

int DiffusionSolver::read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) {
  (void)solvers;
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty() || line[0] == "}") break;
    bool used = false;
    PG_TRY(readCommon(line, tok, mesh, used), "wrong solver block");
    PG_CHECK(!used, "unrecognized keyword '" + line[0] + "'");
  }
  return 0;
}

namespace {

// math::surface_leakage_factor (math.cxx:150-161).
inline double slf(const double* p1, const double* p2, const double* n) {
  double dp[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
  double num = 0.0, den = 0.0;
  for (int d = 0; d < 3; d++) num += dp[d] * n[d];
  for (int d = 0; d < 3; d++) den += dp[d] * dp[d];
  return num / den;
}

void material_tables(const std::vector<Material>& mats, int G, std::vector<double>& st,
                     std::vector<double>& ss, std::vector<double>& chi, std::vector<double>& nsf,
                     std::vector<double>& ksf) {
  const size_t nm = mats.size();
  st.assign(nm * G, 0.0);
  ss.assign(nm * G * G, 0.0);
  chi.assign(nm * G, 0.0);
  nsf.assign(nm * G, 0.0);
  ksf.assign(nm * G, 0.0);
  for (size_t m = 0; m < nm; m++) {
    if (!mats[m].has_nd) continue;
    for (int g = 0; g < G; g++) {
      st[m * G + g] = mats[m].sigma_t[g];
      chi[m * G + g] = mats[m].chi[g];
      nsf[m * G + g] = mats[m].nu_sigma_f[g];
      ksf[m * G + g] = mats[m].kappa_sigma_f[g];
    }
    for (int k = 0; k < G * G; k++) ss[m * G * G + k] = mats[m].sigma_s[k];
  }
}

}  // namespace

// R of DiffusionSolver::buildMatrices (DiffusionSolver.cxx:88-320, n = 0), cell-stencil
// layout.  The diagonal accumulates in the reference's order: total, self-scatter, then
// each face in turn.
// With feedback nuclear data (T given) every cross section of row i is the material's at
// the temperature of cell i, the neighbour's diffusion coefficient included (the reference
// evaluates both with T_data[i], DiffusionSolver.cxx:250-279); "same material" still
// compares the materials themselves.
int assemble_diffusion(const Mesh& mesh, const std::vector<Material>& mats, int G,
                       const std::map<int, BoundaryCondition>& bcs, std::vector<int>& neighbors,
                       std::vector<double>& offdiag, std::vector<double>& diag, const std::vector<double>* T) {
  const int n = mesh.num_cells, F = mesh.fmax;
  neighbors.assign((size_t)F * n, -1);
  offdiag.assign((size_t)F * n * G, 0.0);
  diag.assign((size_t)n * G, 0.0);
  std::map<std::pair<int, double>, Material> at_T;
  auto data = [&](int m, int cell) -> const Material& {
    if (!T || !mats[m].feedback()) return mats[m];
    const double t = (*T)[cell];
    auto it = at_T.find({m, t});
    if (it == at_T.end()) {
      Material md;
      mats[m].at(t, md);
      it = at_T.emplace(std::make_pair(m, t), md).first;
    }
    return it->second;
  };
  for (int i = 0; i < n; i++) {
    const Material& mat = data(mesh.materials[i], i);
    const double V = mesh.volumes[i];
    for (int f = 0; f < mesh.num_faces[i]; f++) {
      int i2 = mesh.nbr(i, f);
      if (i2 >= 0) neighbors[(size_t)f * n + i] = i2;
    }
    for (int g = 0; g < G; g++) {
      double d = mat.sigma_t[g] * V;
      d += -mat.sigma_s[(size_t)g * G + g] * V;
      for (int f = 0; f < mesh.num_faces[i]; f++) {
        const int i2 = mesh.nbr(i, f);
        const double A = mesh.area(i, f);
        if (i2 < 0) {
          auto it = bcs.find(-i2);
          BCType type = it == bcs.end() ? BC_NONE : it->second.type;
          if (type == BC_VACUUM) {
            double w = slf(mesh.cc(i), mesh.fc(i, f), mesh.nrm(i, f));
            d += w * mat.diffusion[g] * A;
          } else if (type == BC_REFLECTIVE) {
          } else if (type == BC_ROBIN) {
            d -= it->second.values.at(0) * A;
          } else {
            PG_CHECK(true, "boundary condition not implemented");
          }
          continue;
        }
        const Material& mat2 = data(mesh.materials[i2], i);
        double r;
        if (mesh.materials[i2] == mesh.materials[i]) {
          double w = slf(mesh.cc(i), mesh.cc(i2), mesh.nrm(i, f));
          r = -w * mat.diffusion[g] * A;
        } else {
          double w1 = slf(mesh.cc(i), mesh.fc(i, f), mesh.nrm(i, f));
          w1 *= mat.diffusion[g] * A;
          double w2 = slf(mesh.cc(i2), mesh.fc(i, f), mesh.nrm(i, f));
          w2 *= -mat2.diffusion[g] * A;
          r = -(w1 * w2) / (w1 + w2);
        }
        d -= r;
        offdiag[((size_t)f * n + i) * G + g] = r;
      }
      diag[(size_t)i * G + g] = d;
    }
  }
  return 0;
}

int DiffusionSolver::buildProblem() {
  const Mesh& mesh = *mesh_;
  std::vector<int> nbr;
  std::vector<double> off, diag, st, ss, chi, nsf, ksf;
  PG_TRY(assemble_diffusion(mesh, *mats_, G_, boundaryConditions(), nbr, off, diag, feedback_ ? &T_ : nullptr),
         "unable to assemble the diffusion operator");
  material_tables(cell_mats_, G_, st, ss, chi, nsf, ksf);
  pgpu_diffusion_operator op;
  op.num_cells = mesh.num_cells;
  op.num_groups = G_;
  op.num_faces = mesh.fmax;
  op.num_materials = (int)cell_mats_.size();
  op.neighbors = nbr.data();
  op.offdiag = off.data();
  op.diag = diag.data();
  op.materials = cell_mat_.data();
  op.volumes = mesh.volumes.data();
  op.sigma_s = ss.data();
  op.chi = chi.data();
  op.nu_sigma_f = nsf.data();
  op.kappa_sigma_f = ksf.data();
  int st_code = pgpu_diffusion_create(opt_.device, &op, &problem_);
  PG_CHECK(st_code != PGPU_OK, std::string("unable to upload the operator: ") + pgpu_last_error());
  return 0;
}

int DiffusionSolver::fetchSolution() { return 0; }

DiffusionSolver::~DiffusionSolver() {
  if (transient_problem_) pgpu_problem_destroy(transient_problem_);
}

int DiffusionSolver::finalize() {
  if (transient_problem_) pgpu_problem_destroy(transient_problem_);
  transient_problem_ = nullptr;
  return NeutronicSolver::finalize();
}

// Transient step n > 0 of DiffusionSolver (DiffusionSolver.cxx:94-175, getSolution :337-345):
// keep the previous step's flux as phi0 when the step advances, then solve
//   (R + V/(v dt) - (1 - beta) chi_p nu_sigma_f V / keff) phi = chi_d S + V/(v dt) phi0
// on the GPU (pgpu_problem_solve_linear), starting from the current flux as the
// reference's KSP does (petsc.cxx:168), and compute the power, the production rate and the
// delayed source S = beta P (NeutronicSolver.cxx:81-116).
int DiffusionSolver::solveTransient(int n, double dt, double t) {
  (void)t;
  PG_CHECK(keff_ <= 0.0, "the steady state must be solved before a transient step");
  PG_CHECK(!(dt > 0.0), "wrong time-step size");
  const Mesh& mesh = *mesh_;
  const int nc = mesh.num_cells;
  if (n > n0_ + 1) {
    phi_prev_ = phi_;
    n0_++;
  }
  if (!transient_problem_ || dt != transient_dt_ || temperatureChanged()) {
    if (transient_problem_) pgpu_problem_destroy(transient_problem_);
    transient_problem_ = nullptr;
    buildCellMaterials();
    std::vector<int> nbr;
    std::vector<double> off, diag, st, ss, chi, nsf, ksf;
    PG_TRY(assemble_diffusion(mesh, *mats_, G_, boundaryConditions(), nbr, off, diag, feedback_ ? &T_ : nullptr),
           "unable to assemble the diffusion operator");
    material_tables(cell_mats_, G_, st, ss, chi, nsf, ksf);
    for (int i = 0; i < nc; i++) {
      const Material& mat = cell_mats_[cell_mat_[i]];
      for (int g = 0; g < G_; g++) diag[(size_t)i * G_ + g] += mesh.volumes[i] / (mat.velocity[g] * dt);
    }
    for (size_t m = 0; m < cell_mats_.size(); m++) {
      const Material& mat = cell_mats_[m];
      if (!mat.has_nd) continue;
      for (int g = 0; g < G_; g++) chi[m * G_ + g] = (1.0 - mat.beta_total) * mat.chi_prompt[g];
    }
    pgpu_diffusion_operator op;
    op.num_cells = nc;
    op.num_groups = G_;
    op.num_faces = mesh.fmax;
    op.num_materials = (int)cell_mats_.size();
    op.neighbors = nbr.data();
    op.offdiag = off.data();
    op.diag = diag.data();
    op.materials = cell_mat_.data();
    op.volumes = mesh.volumes.data();
    op.sigma_s = ss.data();
    op.chi = chi.data();
    op.nu_sigma_f = nsf.data();
    op.kappa_sigma_f = ksf.data();
    int code = pgpu_diffusion_create(opt_.device, &op, &transient_problem_);
    PG_CHECK(code != PGPU_OK, std::string("unable to upload the transient operator: ") + pgpu_last_error());
    transient_dt_ = dt;
  }
  std::vector<double> b((size_t)nc * G_);
  for (int i = 0; i < nc; i++) {
    const Material& mat = cell_mats_[cell_mat_[i]];
    for (int g = 0; g < G_; g++) {
      const size_t l = (size_t)i * G_ + g;
      b[l] = mat.chi_delayed[g] * S_[i] + mesh.volumes[i] / (mat.velocity[g] * dt) * phi_prev_[l];
    }
  }
  int st = pgpu_problem_solve_linear(transient_problem_, 1.0 / keff_, b.data(), phi_.data(), &opt_.gpu, &stats_);
  PG_CHECK(st != PGPU_OK, std::string("GPU transient solve failed: ") + pgpu_last_error());
  powerAndProduction();
  return 0;
}

// ----------------------------------------------------------------------------------
// SN
// ----------------------------------------------------------------------------------

int SNSolver::read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) {
  (void)solvers;
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty() || line[0] == "}") break;
    bool used = false;
    PG_TRY(readCommon(line, tok, mesh, used), "wrong solver block");
    if (used) continue;
    const std::string& k = line[0];
    PG_CHECK(line.size() != 2, "wrong number of arguments for keyword '" + k + "'");
    if (k == "order") {
      PG_TRY(to_int(line[1], 1, INT_MAX, order_), "wrong SN order");
    } else if (k == "mixed-face-interpolation") {
      PG_TRY(to_double(line[1], 0.0, 1.0, delta_), "wrong weight between upwind and linear interpolation");
    } else if (k == "least-squares-boundary-interpolation") {
      PG_TRY(to_bool(line[1], ls_), "wrong switch for least-squares boundary interpolation");
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  return 0;
}

// Level-symmetric S2..S8 sets (AngularQuadratureSet.cxx:4-209): first-octant cosines and
// weights/8, mirrored into octant o by negating x, y, z for bits 0, 1, 2 of o; the
// reflected direction about each axis is the one whose dot product with the mirror
// image exceeds 1 - 1e-6.
int build_quadrature(int order, std::vector<double>& dirs, std::vector<double>& w,
                     std::vector<int>& refl) {
  const int M = order * (order + 2);
  dirs.assign((size_t)M * 3, 0.0);
  w.assign(M, 0.0);
  auto set = [&](int m, double a, double b, double c) {
    dirs[m * 3] = a;
    dirs[m * 3 + 1] = b;
    dirs[m * 3 + 2] = c;
  };
  if (order == 2) {
    const double s = 1.0 / std::sqrt(3.0);
    set(0, s, s, s);
    w[0] = 1.0 / 8.0;
  } else if (order == 4) {
    const double a = 0.3500212, b = 0.8688903;
    set(0, a, a, b); set(1, a, b, a); set(2, b, a, a);
    for (int m = 0; m < 3; m++) w[m] = (1.0 / 3.0) / 8.0;
  } else if (order == 6) {
    const double a = 0.2666355, b = 0.6815076, c = 0.9261808;
    set(0, a, a, c); set(1, a, c, a); set(2, c, a, a);
    set(3, a, b, b); set(4, b, a, b); set(5, b, b, a);
    for (int m = 0; m < 3; m++) w[m] = 0.1761263 / 8.0;
    for (int m = 3; m < 6; m++) w[m] = 0.1572071 / 8.0;
  } else if (order == 8) {
    const double a = 0.2182179, b = 0.5773503, c = 0.7867958, d = 0.9511897;
    set(0, a, a, d); set(1, a, d, a); set(2, d, a, a);
    set(3, a, b, c); set(4, a, c, b); set(5, b, a, c);
    set(6, b, c, a); set(7, c, a, b); set(8, c, b, a); set(9, b, b, b);
    for (int m = 0; m < 3; m++) w[m] = 0.1209877 / 8.0;
    for (int m = 3; m < 9; m++) w[m] = 0.0907407 / 8.0;
    w[9] = 0.0925926 / 8.0;
  } else {
    PG_CHECK(true, "SN order not implemented");
  }
  const int m8 = M / 8;
  for (int o = 1; o < 8; o++)
    for (int m = 0; m < m8; m++) {
      int l = o * m8 + m;
      dirs[l * 3 + 0] = (o & 1) ? -dirs[m * 3 + 0] : dirs[m * 3 + 0];
      dirs[l * 3 + 1] = (o & 2) ? -dirs[m * 3 + 1] : dirs[m * 3 + 1];
      dirs[l * 3 + 2] = (o & 4) ? -dirs[m * 3 + 2] : dirs[m * 3 + 2];
      w[l] = w[m];
    }
  refl.assign((size_t)M * 3, -1);
  for (int a = 0; a < 3; a++)
    for (int m = 0; m < M; m++) {
      double r[3];
      double dd = -2.0 * dirs[m * 3 + a];
      for (int k = 0; k < 3; k++) r[k] = (k == a ? dd : 0.0) + dirs[m * 3 + k];
      for (int m2 = 0; m2 < M; m2++) {
        double dot = dirs[m2 * 3] * r[0] + dirs[m2 * 3 + 1] * r[1] + dirs[m2 * 3 + 2] * r[2];
        if (dot > 1.0 - 1.0e-6) {
          PG_CHECK(refl[m * 3 + a] != -1, "multiple reflected directions found");
          refl[m * 3 + a] = m2;
        }
      }
      PG_CHECK(refl[m * 3 + a] == -1, "reflected direction not found");
    }
  return 0;
}

namespace {

inline double dist3(const double* a, const double* b) {
  double s = 0.0;
  for (int d = 0; d < 3; d++) s += std::pow(b[d] - a[d], 2);
  return std::sqrt(s);
}

// 3x3 (or smaller) inverse by Gauss-Jordan with partial pivoting.
int small_inverse(int n, const double* A, double* Ainv) {
  double a[3][6];
  for (int r = 0; r < n; r++)
    for (int c = 0; c < 2 * n; c++) a[r][c] = c < n ? A[r * n + c] : (c - n == r ? 1.0 : 0.0);
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
    PG_CHECK(a[p][c] == 0.0, "singular least-squares gradient matrix");
    if (p != c)
      for (int k = 0; k < 2 * n; k++) std::swap(a[p][k], a[c][k]);
    double piv = a[c][c];
    for (int k = 0; k < 2 * n; k++) a[c][k] /= piv;
    for (int r = 0; r < n; r++)
      if (r != c) {
        double f = a[r][c];
        for (int k = 0; k < 2 * n; k++) a[r][k] -= f * a[c][k];
      }
  }
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++) Ainv[r * n + c] = a[r][c + n];
  return 0;
}

}  // namespace

int SNSolver::buildProblem() {
  const auto t_start = std::chrono::steady_clock::now();
  psi_solved_ = false;  // a new device problem holds no solution yet
  const Mesh& mesh = *mesh_;
  const int n = mesh.num_cells, F = mesh.fmax, G = G_;
  std::vector<double> dirs, w;
  std::vector<int> refl;
  PG_TRY(build_quadrature(order_, dirs, w, refl), "unable to build the angular quadrature set");
  M_ = (int)w.size();
  const auto& bcs = boundaryConditions();

  std::vector<int> kind((size_t)F * n, PGPU_FACE_NONE), nbr((size_t)F * n, -1),
      raxis((size_t)F * n, -1);
  std::vector<double> area((size_t)F * n, 0.0), nrm((size_t)F * n * 3, 0.0),
      gauss((size_t)F * n * 4, 0.0);
  std::vector<double> lsw;
  bool any_reflective = false;
  for (int i = 0; i < n; i++)
    for (int f = 0; f < mesh.num_faces[i]; f++) {
      const size_t o = (size_t)f * n + i;
      const int i2 = mesh.nbr(i, f);
      area[o] = mesh.area(i, f);
      for (int d = 0; d < 3; d++) nrm[o * 3 + d] = mesh.nrm(i, f)[d];
      if (i2 >= 0) {
        kind[o] = PGPU_FACE_INTERIOR;
        nbr[o] = i2;
        // SNSolver::buildGaussGradientScheme (SNSolver.cxx:159-208)
        double r_if = dist3(mesh.fc(i, f), mesh.cc(i));
        double r_i2f = dist3(mesh.fc(i, f), mesh.cc(i2));
        double r_ii2 = dist3(mesh.cc(i), mesh.cc(i2));
        gauss[o * 4 + 0] = (r_i2f + delta_ * r_if) / r_ii2;
        gauss[o * 4 + 1] = (1.0 - delta_) * r_if / r_ii2;
        gauss[o * 4 + 2] = (1.0 - delta_) * r_i2f / r_ii2;
        gauss[o * 4 + 3] = (r_if + delta_ * r_i2f) / r_ii2;
      } else {
        auto it = bcs.find(-i2);
        BCType type = it == bcs.end() ? BC_NONE : it->second.type;
        if (type == BC_VACUUM) {
          kind[o] = PGPU_FACE_VACUUM;
        } else if (type == BC_REFLECTIVE) {
          kind[o] = PGPU_FACE_REFLECTIVE;
          any_reflective = true;
          // SNSolver.cxx:539-543: the axis loop variable shadows the cell index, so face
          // f of cells 0, 1 and 2 is tested against the x, y and z axes respectively.
          int axis = -1;
          for (int a = 0; a < 3; a++) {
            const int ca = a < n ? a : i;
            if (f >= mesh.num_faces[ca]) continue;
            double dd = mesh.nrm(ca, f)[a];
            if (std::fabs(dd) > 1.0 - 1.0e-6) axis = a;
          }
          PG_CHECK(axis < 0, "reflected direction not found");
          raxis[o] = axis;
        } else {
          PG_CHECK(true, "boundary condition not implemented");
        }
      }
    }
  (void)any_reflective;
  if (ls_) {
    // SNSolver::buildLSGradientScheme (SNSolver.cxx:211-269) for cells with a boundary
    // face, then the vacuum-face correction weights dp_f . c_f2 (SNSolver.cxx:486-513).
    // As in the reference, d(jg, f) reads the flat element jg*dims + f of the
    // (faces x dims) array, and the Gram matrix starts from zero.
    const int nd = mesh.num_dims;
    PG_CHECK(nd < 1 || nd > 3, "wrong number of dimensions for the LS gradient");
    lsw.assign((size_t)F * n * F, 0.0);
    for (int i = 0; i < n; i++) {
      const int nf = mesh.num_faces[i];
      bool bcell = false;
      for (int f = 0; f < nf; f++) bcell |= mesh.nbr(i, f) < 0;
      if (!bcell) continue;
      std::vector<double> d((size_t)nf * nd);
      for (int f = 0; f < nf; f++) {
        int i2 = mesh.nbr(i, f);
        const double* c2 = i2 < 0 ? mesh.fc(i, f) : mesh.cc(i2);
        for (int a = 0; a < nd; a++) d[(size_t)f * nd + a] = c2[a] - mesh.cc(i)[a];
      }
      auto flat = [&](int r, int c) { return d[(size_t)r * nd + c]; };  // d(r, c) of the reference
      double Gm[9] = {0}, Gi[9];
      for (int jg = 0; jg < nd; jg++)
        for (int ig = 0; ig < nd; ig++)
          for (int f = 0; f < nf; f++) Gm[jg * nd + ig] += flat(jg, f) * flat(f, ig);
      PG_TRY(small_inverse(nd, Gm, Gi), "unable to invert the LS gradient matrix");
      std::vector<double> c((size_t)nf * 3, 0.0);
      for (int f = 0; f < nf; f++)
        for (int a = 0; a < nd; a++)
          for (int b = 0; b < nd; b++) c[(size_t)f * 3 + a] += Gi[a * nd + b] * flat(b, f);
      for (int f = 0; f < nf; f++) {
        if (kind[(size_t)f * n + i] != PGPU_FACE_VACUUM) continue;
        double dp[3];
        for (int a = 0; a < 3; a++) dp[a] = mesh.fc(i, f)[a] - mesh.cc(i)[a];
        for (int f2 = 0; f2 < nf; f2++) {
          if (mesh.nbr(i, f2) < 0) continue;
          lsw[((size_t)f * n + i) * F + f2] =
              dp[0] * c[(size_t)f2 * 3] + dp[1] * c[(size_t)f2 * 3 + 1] + dp[2] * c[(size_t)f2 * 3 + 2];
        }
      }
    }
  }
  std::vector<double> st, ss, chi, nsf, ksf;
  material_tables(cell_mats_, G, st, ss, chi, nsf, ksf);
  pgpu_sn_operator op;
  std::memset(&op, 0, sizeof(op));
  op.num_cells = n;
  op.num_groups = G;
  op.num_dirs = M_;
  op.num_faces = F;
  op.num_materials = (int)cell_mats_.size();
  op.use_ls = ls_ ? 1 : 0;
  op.num_cell_faces = mesh.num_faces.data();
  op.face_kind = kind.data();
  op.neighbors = nbr.data();
  op.areas = area.data();
  op.normals = nrm.data();
  op.gauss = gauss.data();
  op.reflect_axis = raxis.data();
  op.ls_weight = ls_ ? lsw.data() : nullptr;
  op.materials = cell_mat_.data();
  op.volumes = mesh.volumes.data();
  op.directions = dirs.data();
  op.weights = w.data();
  op.reflected = refl.data();
  op.sigma_t = st.data();
  op.sigma_s = ss.data();
  op.chi = chi.data();
  op.nu_sigma_f = nsf.data();
  op.kappa_sigma_f = ksf.data();
  op.cart_nx = mesh.cart_nx;
  op.cart_ny = mesh.cart_ny;
  op.cart_nz = mesh.cart_nz;
  const auto t_assembled = std::chrono::steady_clock::now();
  int code = pgpu_sn_create(opt_.device, &op, &problem_);
  PG_CHECK(code != PGPU_OK, std::string("unable to upload the SN operator: ") + pgpu_last_error());
  if (std::getenv("PGPU_HOST_TIMING")) {  // measurement: host assembly and device setup of the operator
    const auto t_end = std::chrono::steady_clock::now();
    std::fprintf(stderr, "pgpu host: SN assembly %.3f s, pgpu_sn_create %.3f s\n",
                 std::chrono::duration<double>(t_assembled - t_start).count(),
                 std::chrono::duration<double>(t_end - t_assembled).count());
  }
  return 0;
}

int SNSolver::initialize(const Mesh& mesh, const std::vector<Material>& mats,
                         const RunOptions& opt, bool transient) {
  PG_TRY(NeutronicSolver::initialize(mesh, mats, opt, transient), "unable to initialize");
  PG_CHECK(order_ != 2 && order_ != 4 && order_ != 6 && order_ != 8, "SN order not implemented");
  M_ = order_ * (order_ + 2);
  // SNSolver.cxx:745-747; zero until the first solve, as the reference's new vector
  const size_t N = (size_t)mesh.num_cells * G_ * M_;
  psi_.clear();
  psi_host_ = psi_solved_ = false;
  Field f{"angular-flux", nullptr, false, false, nullptr};
  f.size = N;
  f.get = [this, N](double* v) -> int {
    if (psi_host_) {
      std::memcpy(v, psi_.data(), N * sizeof(double));
    } else if (psi_solved_ && problem_) {
      PG_TRY(pgpu_problem_get_angular_flux(problem_, v), "unable to get the angular flux");
    } else {
      std::memset(v, 0, N * sizeof(double));
    }
    return 0;
  };
  f.set = [this, N](const double* v) -> int {
    psi_.assign(v, v + N);
    psi_host_ = true;
    return 0;
  };
  fields_.push_back(f);
  return 0;
}

int SNSolver::fetchSolution() {
  psi_solved_ = true;
  psi_host_ = false;
  if (opt_.vtk || opt_.dump) {  // the outputs write the angular flux from the host
    psi_.resize((size_t)mesh_->num_cells * G_ * M_);
    PG_TRY(pgpu_problem_get_angular_flux(problem_, psi_.data()), "unable to get the angular flux");
    psi_host_ = true;
  }
  return 0;
}

}  // namespace pg

namespace pg {

// SNSolver::writeVTK and writePETSc (SNSolver.cxx:753-780).
int SNSolver::writeFields(int n) const {
  const int nc = mesh_->num_cells;
  PG_TRY(write_vtk_field("./output", n, opt_, "flux", phi_, nc, G_), "unable to write the scalar flux");
  PG_TRY(write_vtk_field("./output", n, opt_, "flux", psi_, nc, G_, M_), "unable to write the angular flux");
  PG_TRY(write_vtk_field("./output", n, opt_, "power", q_, nc), "unable to write the thermal power");
  PG_TRY(write_petsc_vec("angular_flux", n, opt_, psi_), "unable to write the angular flux");
  return 0;
}

}  // namespace pg
