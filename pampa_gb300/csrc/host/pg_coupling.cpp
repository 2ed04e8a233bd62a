// Multiphysics pieces of the neutronics path beside the eigen-solve: convergence errors
// (ConvergenceError.hxx), the delayed-neutron precursor solver (PrecursorSolver.cxx) and
// the fixed-point coupling of several solvers (CouplingSolver.cxx).  The neutronic solves
// they drive run on the GPU; what is here is per-cell bookkeeping and field copies.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <iomanip>
#include <iostream>
#include <sstream>

#include "pg_host.hpp"

namespace pg {

// ConvergenceError::check (ConvergenceError.hxx:50-95).
int ConvergenceError::check(const std::vector<double>& v, bool& converged, bool verbose) {
  if (!have_prev_) {
    converged = false;
    if (verbose) std::cout << "Convergence initialized for " << name_ << " vector." << std::endl;
  } else {
    PG_CHECK(prev_.size() != v.size(), "field size changed between coupling iterations");
    double eps = 0.0, nrm = 0.0;
    for (size_t k = 0; k < v.size(); k++) {
      const double d = std::fabs(v[k] - prev_[k]);
      if (norm_ == 1) eps += d;
      else if (norm_ == 2) eps += d * d;
      else eps = std::max(eps, d);
      nrm += v[k] * v[k];
    }
    if (norm_ == 2) eps = std::sqrt(eps);
    if (relative_) eps /= std::sqrt(nrm);
    converged = eps < tol_;
    if (verbose) {
      std::ostringstream msg;
      msg << std::scientific << std::setprecision(3) << "Convergence error for " << name_ << " vector: " << eps
          << (eps > tol_ ? " > " : " < ") << tol_ << (eps > tol_ ? " (not converged)." : " (converged).");
      std::cout << msg.str() << std::endl;
    }
  }
  prev_ = v;
  have_prev_ = true;
  return 0;
}

int read_convergence(const std::vector<std::string>& line, size_t i, std::shared_ptr<ConvergenceError>& out) {
  PG_CHECK(line.size() < i + 4, "wrong number of arguments for a convergence error");
  const std::string& p = line[i + 1];
  int norm;
  if (p == "1") norm = 1;
  else if (p == "2") norm = 2;
  else if (p == "max") norm = 0;
  else PG_CHECK(true, "wrong convergence norm type");
  bool relative = false;
  PG_TRY(to_bool(line[i + 2], relative), "wrong switch for relative convergence");
  double tol = 0.0;
  PG_TRY(to_double(line[i + 3], 0.0, DBL_MAX, tol), "wrong convergence tolerance");
  out = std::make_shared<ConvergenceError>(line[i], norm, relative, tol);
  return 0;
}

// ----------------------------------------------------------------------------------
// PrecursorSolver (PrecursorSolver.cxx:4-202)
// ----------------------------------------------------------------------------------

int PrecursorSolver::read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) {
  (void)mesh;
  (void)solvers;
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty() || line[0] == "}") break;
    const std::string& k = line[0];
    if (k == "precursor-groups") {
      PG_CHECK(line.size() != 2, "wrong number of arguments for keyword '" + k + "'");
      PG_TRY(to_int(line[1], 1, INT_MAX, npg_), "wrong number of delayed-neutron precursor groups");
    } else if (k == "convergence") {
      PG_CHECK(line.size() != 5, "wrong number of arguments for keyword '" + k + "'");
      if (line[1] == "precursors") {
        PG_TRY(read_convergence(line, 1, dC_), "wrong convergence error");
      } else if (line[1] == "delayed-source") {
        PG_TRY(read_convergence(line, 1, dS_), "wrong convergence error");
      } else {
        PG_CHECK(true, "wrong field");
      }
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  return 0;
}

// checkMaterials + build (PrecursorSolver.cxx:132-180): the production rate starts uniform
// with a 1-norm of 1 (petsc::normalize, petsc.cxx:276-287).
int PrecursorSolver::initialize(const Mesh& mesh, const std::vector<Material>& mats, const RunOptions& opt,
                                bool transient) {
  (void)transient;
  mesh_ = &mesh;
  mats_ = &mats;
  opt_ = opt;
  n0_ = -1;
  PG_CHECK(npg_ < 1, "missing number of delayed-neutron precursor groups");
  for (const auto& m : mats)
    if (m.has_pd) PG_CHECK(m.num_precursor_groups != npg_, "wrong precursor data");
  const int n = mesh.num_cells;
  P_.assign(n, 1.0 / n);
  C_.assign((size_t)n * npg_, 0.0);
  C0_.clear();
  S_.assign(n, 0.0);
  fields_.clear();
  fields_.push_back({"production-rate", &P_, true, false, nullptr});
  fields_.push_back({"precursors", &C_, false, true, dC_});
  fields_.push_back({"delayed-source", &S_, false, true, dS_});
  return 0;
}

int PrecursorSolver::solve(int n, double dt, double t) {
  (void)t;
  const int nc = mesh_->num_cells;
  if (n > n0_ + 1) {
    C0_ = C_;
    n0_++;
  }
  for (int i = 0; i < nc; i++) {
    const Material& m = (*mats_)[mesh_->materials[i]];
    S_[i] = 0.0;
    if (!m.has_pd) continue;
    for (int g = 0; g < npg_; g++) {
      const size_t l = (size_t)i * npg_ + g;
      const double beta = m.precursor_beta[g], lambda = m.precursor_lambda[g];
      C_[l] = n == 0 ? (beta / lambda) * P_[i] : (C0_[l] + dt * beta * P_[i]) / (1.0 + dt * lambda);
      S_[i] += lambda * C_[l];
    }
  }
  return 0;
}

// printLog (PrecursorSolver.cxx:183-192).
int PrecursorSolver::output(int n, bool write_mesh) const {
  if (!opt_.silent) {
    double cmin = C_.empty() ? 0.0 : *std::min_element(C_.begin(), C_.end());
    double cmax = C_.empty() ? 0.0 : *std::max_element(C_.begin(), C_.end());
    std::cout << std::scientific << std::setprecision(3) << "Precursor population: " << cmin << " (min), " << cmax
              << " (max)." << std::endl;
  }
  // writeVTK and writePETSc (PrecursorSolver.cxx:195-215)
  if (write_mesh) PG_TRY(write_vtk_mesh("./output", n, opt_, *mesh_), "unable to write the mesh in .vtk format");
  PG_TRY(write_vtk_field("./output", n, opt_, "precursor", C_, mesh_->num_cells, npg_),
         "unable to write the precursor population");
  PG_TRY(write_petsc_vec("precursors", n, opt_, C_), "unable to write the precursor population");
  return 0;
}

// ----------------------------------------------------------------------------------
// CouplingSolver (CouplingSolver.cxx:4-174)
// ----------------------------------------------------------------------------------

int CouplingSolver::read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) {
  (void)mesh;
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty() || line[0] == "}") break;
    const std::string& k = line[0];
    if (k == "coupled-solvers") {
      PG_CHECK(line.size() < 2, "wrong number of arguments for keyword '" + k + "'");
      int num = 0;
      PG_TRY(to_int(line[1], 1, INT_MAX, num), "wrong number of coupled solvers");
      PG_CHECK(line.size() != (size_t)(2 + num), "wrong number of arguments for keyword '" + k + "'");
      coupled_.clear();
      for (int c = 0; c < num; c++) {
        Solver* found = nullptr;
        for (Solver* s : solvers)
          if (s->name() == line[2 + c]) found = s;
        PG_CHECK(!found, "unable to find the coupled solver");
        coupled_.push_back(found);
      }
    } else if (k == "implicit") {
      PG_CHECK(line.size() != 2, "wrong number of arguments for keyword '" + k + "'");
      PG_TRY(to_bool(line[1], implicit_), "wrong switch for implicit coupling");
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  return 0;
}

int CouplingSolver::initialize(const Mesh& mesh, const std::vector<Material>& mats, const RunOptions& opt,
                               bool transient) {
  opt_ = opt;
  mesh_ = &mesh;
  PG_CHECK(coupled_.empty(), "no coupled solvers");
  for (Solver* s : coupled_) PG_TRY(s->initialize(mesh, mats, opt, transient), "unable to initialize the solver");
  fields_.clear();
  for (Solver* s : coupled_)
    for (const Field& f : s->fields()) fields_.push_back(f);
  return 0;
}

int CouplingSolver::solve(int n, double dt, double t) {
  const bool verbose = opt_.verbose && !opt_.silent;
  bool converged = false;
  for (int it = 0; !converged; it++) {
    PG_CHECK(it >= kMaxCouplingIterations, "the coupled solution did not converge");
    converged = true;
    for (size_t i = 0; i < coupled_.size(); i++) {
      PG_TRY(coupled_[i]->solve(n, dt, t), "unable to get the solution");
      for (Field& out : coupled_[i]->fields()) {
        if (!out.output) continue;
        for (size_t i2 = 0; i2 < coupled_.size(); i2++) {
          if (i2 == i) continue;
          for (Field& in : coupled_[i2]->fields()) {
            if (!in.input || in.name != out.name) continue;
            PG_CHECK(in.vec->size() != out.vec->size(), "field sizes differ between coupled solvers");
            *in.vec = *out.vec;
            if (verbose)
              std::cout << "Feedback performed for " << out.name << " vector (" << coupled_[i]->name() << " -> "
                        << coupled_[i2]->name() << ")." << std::endl;
          }
        }
        if (implicit_) {
          PG_CHECK(!out.delta, "missing convergence error for the " + out.name + " field");
          bool conv = false;
          PG_TRY(out.delta->check(*out.vec, conv, verbose), "unable to check the convergence");
          converged &= conv;
        }
      }
    }
    if (verbose)
      std::cout << (converged ? "Coupled solution converged." : "Coupled solution not converged.") << std::endl;
  }
  return 0;
}

// CouplingSolver::output (CouplingSolver.cxx:148-163): the mesh once, then every coupled
// solver's summary and fields.
int CouplingSolver::output(int n, bool write_mesh) const {
  if (write_mesh) PG_TRY(write_vtk_mesh("./output", n, opt_, *mesh_), "unable to write the mesh in .vtk format");
  for (Solver* s : coupled_) PG_TRY(s->output(n, false), "unable to output the solution");
  return 0;
}

int CouplingSolver::finalize() {
  for (Solver* s : coupled_) PG_TRY(s->finalize(), "unable to finalize the solver");
  return 0;
}

NeutronicSolver* CouplingSolver::neutronic() {
  for (Solver* s : coupled_)
    if (NeutronicSolver* ns = s->neutronic()) return ns;
  return nullptr;
}

}  // namespace pg
