// Host-side model of pampa's steady-state neutronics path: input tokens, materials,
// meshes and the solver classes behind the drop-in C API.  Everything here is plain
// C++17; the arithmetic of the solve lives in the CUDA kernels behind pgpu_*.
#pragma once

#include <cstdio>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "pampa_gb300.h"

namespace pg {

// Error convention of the reference (utils.hxx:41-47): print "file:line:func(): error:
// message." and return 1.
#define PG_CHECK(cond, msg)                                                              \
  do {                                                                                   \
    if (cond) {                                                                          \
      std::printf("%s:%d:%s(): error: %s.\n", __FILE__, __LINE__, __func__,             \
                  std::string(msg).c_str());                                             \
      std::fflush(stdout);                                                               \
      return 1;                                                                          \
    }                                                                                    \
  } while (0)

#define PG_TRY(call, msg) PG_CHECK((call) != 0, msg)

// ----------------------------------------------------------------------------------
// Tokens: line reader with the semantics of input::get_next_line (input.cxx:4-62).
// ----------------------------------------------------------------------------------
class Tokens {
 public:
  int open(const std::string& path);
  std::vector<std::string> next();
  int read_doubles(std::vector<double>& v, size_t n, double lo, double hi);
  int read_ints(std::vector<int>& v, size_t n, int lo, int hi);
  const std::string& path() const { return path_; }

 private:
  std::string path_;
  std::vector<std::string> lines_;
  size_t pos_ = 0;
};

int to_int(const std::string& s, int lo, int hi, int& out);
int to_double(const std::string& s, double lo, double hi, double& out);
int to_bool(const std::string& s, bool& out);
std::string resolve_path(const std::string& path, const std::string& base_dir);

// ----------------------------------------------------------------------------------
// Boundary conditions (utils.hxx:96-117).
// ----------------------------------------------------------------------------------
enum BCType { BC_NONE = 0, BC_VACUUM, BC_REFLECTIVE, BC_ROBIN, BC_DIRICHLET, BC_ADIABATIC,
              BC_CONVECTION };

struct BoundaryCondition {
  BCType type = BC_NONE;
  std::vector<double> values;  // steady state: value of each function at t = 0
};

int read_bc(const std::vector<std::string>& line, size_t i, Tokens& tok, BoundaryCondition& bc);

// ----------------------------------------------------------------------------------
// Materials with constant nuclear data (Material.cxx, ConstantNuclearData.cxx).
// ----------------------------------------------------------------------------------
struct Material {
  std::string name;
  bool bc = false, split = false, fuel = false, has_nd = false;
  int num_groups = -1;
  double beta_total = 0.0;
  int num_sub = 0;
  // precursor data (PrecursorData.hxx): groups, decay constants, delayed fractions
  bool has_pd = false;
  int num_precursor_groups = 0;
  std::vector<double> precursor_lambda, precursor_beta;
  std::vector<double> sigma_t, nu_sigma_f, kappa_sigma_f, sigma_tr, diffusion, chi_prompt,
      chi_delayed, chi, velocity;
  std::vector<double> sigma_s;  // [from][to]

  // feedback nuclear data (FeedbackNuclearData.hxx): one constant set per reference
  // temperature, interpolated linearly at a cell's temperature; empty for constant data
  std::vector<double> tref;
  std::vector<Material> feedback_sets;
  bool feedback() const { return !feedback_sets.empty(); }
  // the constant data of this material at temperature T (itself for constant data)
  void at(double T, Material& out) const;

  int read(Tokens& tok);
  int read_file(const std::string& path);
  int check_for_solver(int G, bool diffusion, bool transient = false) const;

 private:
  int read_nuclear_data(Tokens& tok);
  int finish_nuclear_data();
};

// ----------------------------------------------------------------------------------
// Mesh: cells and padded per-face arrays (row-major cell x face).
// ----------------------------------------------------------------------------------
constexpr int NO_FACE = -2147483647;

struct Mesh {
  int num_dims = 0;
  int num_cells = 0;
  int fmax = 0;
  int cart_nx = 0, cart_ny = 0, cart_nz = 0;  // full Cartesian box without void cells, else 0
  std::vector<double> volumes;    // n
  std::vector<double> centroids;  // n*3
  std::vector<int> materials;     // n
  std::vector<int> num_faces;     // n
  std::vector<double> areas;      // n*fmax
  std::vector<double> fcent;      // n*fmax*3
  std::vector<double> normals;    // n*fmax*3
  std::vector<int> neighbors;     // n*fmax: >= 0 cell, < 0 -(boundary+1), NO_FACE pad
  std::vector<std::string> boundaries;
  std::map<int, BoundaryCondition> bcs;  // 1-based boundary index
  bool has_bcs = false;
  // geometry for the .vtk output (Mesh::writeVTK, Mesh.cxx:397-405): point coordinates and
  // each cell's points in the gmsh order the reference builds them in
  std::vector<double> points;                 // num_points*3
  std::vector<int> cell_pts_ptr{0}, cell_pts;  // CSR: cell i owns cell_pts[ptr[i] .. ptr[i+1])

  int nbr(int i, int f) const { return neighbors[(size_t)i * fmax + f]; }
  double area(int i, int f) const { return areas[(size_t)i * fmax + f]; }
  const double* fc(int i, int f) const { return &fcent[((size_t)i * fmax + f) * 3]; }
  const double* nrm(int i, int f) const { return &normals[((size_t)i * fmax + f) * 3]; }
  const double* cc(int i) const { return &centroids[(size_t)i * 3]; }
  void allocate(int n, int F);
};

int read_cartesian_mesh(const std::string& path, Mesh& mesh);
int read_unstructured_mesh(const std::string& path, Mesh& mesh);
int split_materials(Mesh& mesh, std::vector<Material>& materials);
int remove_bc_materials(const Mesh& in, const std::vector<Material>& materials, Mesh& out);

// ----------------------------------------------------------------------------------
// Solvers (Solver.hxx:31-98, PhysicsSolver.hxx, NeutronicSolver.hxx).
// ----------------------------------------------------------------------------------
// ConvergenceError (ConvergenceError.hxx): the norm of the change of a field between two
// coupling iterations, absolute or relative to the field's L2 norm, against a tolerance.
class ConvergenceError {
 public:
  ConvergenceError(std::string name, int norm, bool relative, double tol)
      : name_(std::move(name)), norm_(norm), relative_(relative), tol_(tol) {}
  // converged = false on the first call (no previous iterate), then |v - v_prev| < tol.
  int check(const std::vector<double>& v, bool& converged, bool verbose);

 private:
  std::string name_;
  int norm_;  // 1, 2, or 0 for the max norm
  bool relative_;
  double tol_;
  bool have_prev_ = false;
  std::vector<double> prev_;
};

// `convergence <field> <1|2|max> <relative 0|1> <tol>` (input.cxx:406-425); name is the
// field, line[i] its first argument.
int read_convergence(const std::vector<std::string>& line, size_t i, std::shared_ptr<ConvergenceError>& out);

struct Field {
  std::string name;
  std::vector<double>* vec = nullptr;
  bool input = false, output = false;
  std::shared_ptr<ConvergenceError> delta;  // convergence of an output field (coupling)
  // A field without a host vector (vec == nullptr) whose values stay where the solver
  // keeps them until asked for: its size and the copies out of and into a caller's buffer.
  size_t size = 0;
  std::function<int(double*)> get;
  std::function<int(const double*)> set;
};

struct RunOptions {
  pgpu_options gpu;
  int device = 0;
  bool verbose = false, silent = false;
  // output switches: -vtk / -vtk_interval (vtk.cxx:15-25) or `vtk on [interval]` in the
  // input, -petsc_dump (petsc.cxx:32) or `petsc dump on`
  bool vtk = false, dump = false;
  int vtk_interval = 1;
};

// .vtk and PETSc binary output (vtk.cxx, petsc.cxx:491-511).
int write_vtk_mesh(const std::string& prefix, int n, const RunOptions& opt, const Mesh& mesh);
int write_vtk_field(const std::string& prefix, int n, const RunOptions& opt, const std::string& name,
                    const std::vector<double>& v, int num_cells, int num_groups = 1, int num_directions = 1);
int write_petsc_vec(const std::string& prefix, int n, const RunOptions& opt, const std::vector<double>& v);

class NeutronicSolver;

class Solver {
 public:
  explicit Solver(std::string name) : name_(std::move(name)) {}
  virtual ~Solver() = default;
  // Solver::read (Solver.hxx:31-98): the solver block, with the solvers defined before it
  // (a coupled solver names them).
  virtual int read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) = 0;
  virtual int initialize(const Mesh& mesh, const std::vector<Material>& mats,
                         const RunOptions& opt, bool transient) = 0;
  virtual int solve(int n, double dt, double t) = 0;
  // PhysicsSolver::output (PhysicsSolver.cxx:17-35): the summary on stdout, then the mesh
  // (write_mesh) and the fields in .vtk format and the PETSc dump when switched on
  virtual int output(int n, bool write_mesh = true) const = 0;
  virtual int finalize() = 0;
  // The neutronic solver of this solver's tree (itself, or the first one a coupled solver
  // holds), for the C API's keff / statistics / problem accessors; null if none.
  virtual NeutronicSolver* neutronic() { return nullptr; }
  int getField(double* v, const std::string& name) const;
  int setField(const double* v, const std::string& name);
  int fieldSize(const std::string& name, int& size) const;
  const std::string& name() const { return name_; }
  std::vector<Field>& fields() { return fields_; }

 protected:
  std::string name_;
  std::vector<Field> fields_;
  int n0_ = -1;  // last time step whose solution was kept (Solver.hxx:56)
};

// PrecursorSolver (PrecursorSolver.cxx): delayed-neutron precursor populations per cell and
// precursor group from the production rate, steady state C = beta/lambda P, time step
// C = (C0 + dt beta P) / (1 + dt lambda), and the delayed source S = sum lambda C.  The
// update is a few operations per cell, done on the host next to the coupling loop.
class PrecursorSolver : public Solver {
 public:
  PrecursorSolver() : Solver("precursors") {}
  int read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) override;
  int initialize(const Mesh& mesh, const std::vector<Material>& mats, const RunOptions& opt,
                 bool transient) override;
  int solve(int n, double dt, double t) override;
  int output(int n, bool write_mesh = true) const override;
  int finalize() override { return 0; }

 private:
  const Mesh* mesh_ = nullptr;
  const std::vector<Material>* mats_ = nullptr;
  RunOptions opt_;
  int npg_ = -1;
  const Mesh* mesh_out_ = nullptr;
  // convergence errors of the output fields (PrecursorSolver.hxx:18-22 defaults)
  std::shared_ptr<ConvergenceError> dC_ = std::make_shared<ConvergenceError>("precursors", 2, true, 1.0);
  std::shared_ptr<ConvergenceError> dS_ = std::make_shared<ConvergenceError>("delayed-source", 2, true, 1.0);
  std::vector<double> P_, C_, C0_, S_;
};

// CouplingSolver (CouplingSolver.cxx): fixed-point (Picard) iteration over coupled solvers,
// copying every output field into the solvers that take it as input, until the output
// fields' convergence errors are met (implicit coupling) or once (explicit coupling).
class CouplingSolver : public Solver {
 public:
  explicit CouplingSolver(std::string name) : Solver(std::move(name)) {}
  int read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) override;
  int initialize(const Mesh& mesh, const std::vector<Material>& mats, const RunOptions& opt,
                 bool transient) override;
  int solve(int n, double dt, double t) override;
  int output(int n, bool write_mesh = true) const override;
  int finalize() override;
  NeutronicSolver* neutronic() override;

 private:
  std::vector<Solver*> coupled_;
  bool implicit_ = false;
  RunOptions opt_;
  const Mesh* mesh_ = nullptr;
};

// The reference iterates an implicit coupling until it converges, with no cap; here a
// coupling that has not converged after this many iterations is an error.
constexpr int kMaxCouplingIterations = 1000;

class NeutronicSolver : public Solver {
 public:
  using Solver::Solver;
  ~NeutronicSolver() override;
  int initialize(const Mesh& mesh, const std::vector<Material>& mats, const RunOptions& opt,
                 bool transient) override;
  int solve(int n, double dt, double t) override;
  int output(int n, bool write_mesh = true) const override;
  int finalize() override;
  NeutronicSolver* neutronic() override { return this; }
  double keff() const { return keff_; }
  int problem(pgpu_problem** out);
  const pgpu_stats& stats() const { return stats_; }

 protected:
  int readCommon(const std::vector<std::string>& line, Tokens& tok, const Mesh& mesh, bool& used);
  // convergence errors of the output fields (NeutronicSolver.hxx:39-43 defaults)
  std::shared_ptr<ConvergenceError> dq_ = std::make_shared<ConvergenceError>("power", 2, true, 1.0);
  std::shared_ptr<ConvergenceError> dP_ = std::make_shared<ConvergenceError>("production-rate", 2, true, 1.0);
  virtual int buildProblem() = 0;   // assemble and upload the operator
  virtual int fetchSolution() = 0;  // copy fluxes back after a solve
  // Transient step n > 0 (NeutronicSolver::solve with n > 0, NeutronicSolver.cxx:13-29);
  // solvers without one report an error.
  virtual int solveTransient(int n, double dt, double t);
  // writeVTK / writePETSc of the solver (DiffusionSolver.cxx:410-432, SNSolver.cxx:753-780)
  virtual int writeFields(int n) const;
  void powerAndProduction();        // q, P, S and the total power from phi_ (host)
  void buildCellMaterials();        // cell_mats_ / cell_mat_ at the current temperatures
  bool temperatureChanged() const;  // feedback data and a temperature field changed since
  const std::map<int, BoundaryCondition>& boundaryConditions() const;

  const Mesh* mesh_ = nullptr;
  const std::vector<Material>* mats_ = nullptr;
  RunOptions opt_;
  int G_ = -1;
  double power_ = 1.0;
  std::map<int, BoundaryCondition> bcs_;
  bool has_bcs_ = false;
  double keff_ = -1.0;
  double total_power_ = 0.0;
  std::vector<double> T_, S_, phi_, q_, P_;
  pgpu_problem* problem_ = nullptr;
  pgpu_stats stats_{};
  bool transient_ = false;
  std::vector<double> phi_prev_;     // scalar flux of the previous time step (phi0)
  // the data each cell sees (FeedbackNuclearData at the cell's temperature)
  bool feedback_ = false;
  std::vector<Material> cell_mats_;
  std::vector<int> cell_mat_;
  std::vector<double> T_built_;
};

class DiffusionSolver : public NeutronicSolver {
 public:
  DiffusionSolver() : NeutronicSolver("diffusion") {}
  ~DiffusionSolver() override;
  int read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) override;
  int finalize() override;

 protected:
  int buildProblem() override;
  int fetchSolution() override;
  int solveTransient(int n, double dt, double t) override;
  pgpu_problem* transient_problem_ = nullptr;  // R with the 1/(v dt) terms, chi = (1 - beta) chi_p
  double transient_dt_ = 0.0;
};

class SNSolver : public NeutronicSolver {
 public:
  SNSolver() : NeutronicSolver("sn") {}
  int read(Tokens& tok, const Mesh& mesh, std::vector<Solver*>& solvers) override;
  int initialize(const Mesh& mesh, const std::vector<Material>& mats, const RunOptions& opt,
                 bool transient) override;

 protected:
  int buildProblem() override;
  int fetchSolution() override;
  int writeFields(int n) const override;
  int order_ = -1;
  double delta_ = 0.1;  // SNSolver.hxx:16
  bool ls_ = false;
  int M_ = 0;
  // The angular flux stays on the device: pampa_get_field copies it from there into the
  // caller's buffer.  psi_ holds a host copy only when the .vtk or PETSc outputs need it
  // or a caller set the field (psi_host_); psi_solved_ once the problem holds a solution.
  std::vector<double> psi_;
  bool psi_host_ = false, psi_solved_ = false;
};

// Quadrature of AngularQuadratureSet::build (AngularQuadratureSet.cxx:4-209).
int build_quadrature(int order, std::vector<double>& dirs, std::vector<double>& weights,
                     std::vector<int>& reflected);

// Host assembly into the GPU operator layouts (exposed for tests through the C API).
int assemble_diffusion(const Mesh& mesh, const std::vector<Material>& mats, int G,
                       const std::map<int, BoundaryCondition>& bcs,
                       std::vector<int>& neighbors, std::vector<double>& offdiag,
                       std::vector<double>& diag, const std::vector<double>* T = nullptr);

}  // namespace pg
