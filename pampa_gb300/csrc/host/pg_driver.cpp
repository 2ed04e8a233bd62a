// Parser, Driver and the drop-in C API.
//
// Parser::read (Parser.cxx:4-260): `mesh`, `material`, `solver`, `dt`, `vtk`, `petsc`,
// `include`; before the first solver block, split materials are split and
// boundary-condition materials removed.  Relative file names are tried against the
// working directory first (as the reference does) and then against the directory of the
// file that names them.  Driver (Driver.cxx:4-129) and the pampa_* functions
// (pampa.cxx:5-115) keep the reference's sequence, messages and error convention.
#include <chrono>
#include <climits>
#include <cstring>
#include <iomanip>
#include <iostream>

#include "pg_host.hpp"

namespace pg {

namespace {

std::string dir_of(const std::string& path) {
  size_t p = path.find_last_of('/');
  return p == std::string::npos ? std::string() : path.substr(0, p);
}

struct ParseState {
  std::unique_ptr<Mesh> mesh;
  std::vector<Material> materials;
  std::vector<std::unique_ptr<Solver>> solvers;
  std::vector<double> dt;
  bool ready = false;
  // output switches set by the input (they override the command line)
  bool vtk = false, vtk_set = false, dump = false, dump_set = false;
  int vtk_interval = 1;
};

int parse(const std::string& filename, ParseState& st) {
  Tokens tok;
  PG_TRY(tok.open(filename), "unable to open " + filename);
  const std::string base = dir_of(filename);
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty()) break;
    const std::string& k = line[0];
    if (k == "mesh") {
      PG_CHECK(line.size() != 3, "wrong number of arguments for keyword 'mesh'");
      std::string path = resolve_path(line[2], base);
      st.mesh.reset(new Mesh());
      if (line[1] == "cartesian") {
        PG_TRY(read_cartesian_mesh(path, *st.mesh), "unable to read the mesh from " + path);
      } else if (line[1] == "unstructured") {
        PG_TRY(read_unstructured_mesh(path, *st.mesh), "unable to read the mesh from " + path);
      } else {
        PG_CHECK(true, "mesh type '" + line[1] + "' is not supported by this build");
      }
    } else if (k == "mesh-nodal") {
      PG_CHECK(true, "nodal meshes belong to the heat-conduction solver, not supported here");
    } else if (k == "material") {
      PG_CHECK(line.size() != 3, "wrong number of arguments for keyword 'material'");
      PG_CHECK(!st.mesh, "the mesh must be defined before the materials");
      Material mat;
      mat.name = line[1];
      if (line[2] == "{") {
        PG_TRY(mat.read(tok), "unable to read the material from " + filename);
      } else {
        std::string path = resolve_path(line[2], base);
        PG_TRY(mat.read_file(path), "unable to read the material from " + path);
      }
      if (mat.bc) st.mesh->boundaries.push_back(mat.name);
      st.materials.push_back(mat);
    } else if (k == "solver") {
      PG_CHECK(line.size() < 3, "wrong number of arguments for keyword 'solver'");
      PG_CHECK(!st.mesh, "the mesh must be defined before the solvers");
      if (!st.ready) {
        bool split = false, bc = false;
        for (const auto& m : st.materials) {
          split |= m.split;
          bc |= m.bc;
        }
        if (split) PG_TRY(split_materials(*st.mesh, st.materials), "unable to split materials");
        if (bc) {
          std::unique_ptr<Mesh> m2(new Mesh());
          PG_TRY(remove_bc_materials(*st.mesh, st.materials, *m2),
                 "unable to remove boundary-condition materials from the mesh");
          st.mesh = std::move(m2);
        }
        for (int i = 0; i < st.mesh->num_cells; i++)
          PG_CHECK(st.mesh->materials[i] < 0 || st.mesh->materials[i] >= (int)st.materials.size(),
                   "wrong material index in the mesh");
        st.ready = true;
      }
      // the factory of Parser.cxx:148-165 under the reference's keywords
      std::unique_ptr<Solver> s;
      size_t arg = 2;
      if (line[1] == "diffusion") s.reset(new DiffusionSolver());
      else if (line[1] == "sn") s.reset(new SNSolver());
      else if (line[1] == "precursors") s.reset(new PrecursorSolver());
      else if (line[1] == "coupled") {
        PG_CHECK(line.size() < 4, "wrong number of arguments for keyword 'solver'");
        s.reset(new CouplingSolver(line[2]));
        arg = 3;
      } else {
        PG_CHECK(true, "solver type '" + line[1] + "' is not supported by this build");
      }
      std::vector<Solver*> defined;
      for (auto& d : st.solvers) defined.push_back(d.get());
      if (line[arg] == "{") {
        PG_TRY(s->read(tok, *st.mesh, defined), "unable to read the solver from " + filename);
      } else {
        Tokens t2;
        std::string path = resolve_path(line[arg], base);
        PG_TRY(t2.open(path), "unable to open " + path);
        PG_TRY(s->read(t2, *st.mesh, defined), "unable to read the solver from " + path);
      }
      st.solvers.push_back(std::move(s));
    } else if (k == "dt") {
      PG_CHECK(line.size() != 2, "wrong number of arguments for keyword 'dt'");
      int nt;
      PG_TRY(to_int(line[1], -2147483647, 2147483647, nt), "wrong number of time steps");
      if (nt > 0) {
        PG_TRY(tok.read_doubles(st.dt, nt, 0.0, 1e308), "wrong dt data");
      } else {
        PG_TRY(tok.read_doubles(st.dt, 1, 0.0, 1e308), "wrong dt data");
        st.dt.assign(-nt, st.dt[0]);
      }
    } else if (k == "vtk") {
      // `vtk <switch> [interval]` (Parser.cxx:202-215)
      PG_CHECK(line.size() < 2 || line.size() > 3, "wrong number of arguments for keyword 'vtk'");
      PG_TRY(to_bool(line[1], st.vtk), "wrong switch for .vtk output");
      st.vtk_set = true;
      if (line.size() == 3) PG_TRY(to_int(line[2], 1, INT_MAX, st.vtk_interval), "wrong .vtk output interval");
    } else if (k == "petsc") {
      // `petsc <option> <value>` (Parser.cxx:216-236): dump and verbose are switches; other
      // PETSc/SLEPc solver options have no counterpart on the GPU path
      PG_CHECK(line.size() != 3, "wrong number of arguments for keyword 'petsc'");
      if (line[1] == "dump") {
        PG_TRY(to_bool(line[2], st.dump), "wrong switch to write the solution in PETSc format");
        st.dump_set = true;
      } else if (line[1] == "verbose") {
        bool v = false;
        PG_TRY(to_bool(line[2], v), "wrong switch for verbose PETSc output");
      }
    } else if (k == "include") {
      PG_CHECK(line.size() < 2, "wrong number of arguments for keyword 'include'");
      std::string path = resolve_path(line[1], base);
      PG_TRY(parse(path, st), "unable to parse " + path);
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  return 0;
}

}  // namespace

// Driver (Driver.hxx:13-58): owns the mesh, materials and solvers.
class Driver {
 public:
  int initialize(int argc, char* argv[], std::vector<double>& dt);
  int solve(int n, double dt, double t);
  int finalize();
  Solver* solver() { return solver_; }

 private:
  void print(const std::string& s, bool info = false) const {
    if ((!info || opt_.verbose) && !opt_.silent) std::cout << s << std::endl;
  }
  ParseState st_;
  Solver* solver_ = nullptr;
  RunOptions opt_;
};

int Driver::initialize(int argc, char* argv[], std::vector<double>& dt) {
  PG_CHECK(argc < 2, "missing input file");
  std::string filename(argv[1]);
  opt_ = RunOptions();
  pgpu_default_options(&opt_.gpu);
  for (int a = 2; a < argc; a++) {
    std::string s(argv[a]);
    auto val = [&](void) -> std::string { return a + 1 < argc ? std::string(argv[++a]) : std::string(); };
    if (s == "-verbose") opt_.verbose = true;
    else if (s == "-silent") opt_.silent = true;
    else if (s == "-pgpu_precision") {
      std::string v = val();
      PG_CHECK(v != "fp64" && v != "mixed", "wrong -pgpu_precision (fp64|mixed)");
      opt_.gpu.precision = v == "fp64" ? PGPU_FP64 : PGPU_MIXED;
    } else if (s == "-pgpu_tol_k") PG_TRY(to_double(val(), 0.0, 1.0, opt_.gpu.tol_k), "wrong -pgpu_tol_k");
    else if (s == "-pgpu_tol_flux") PG_TRY(to_double(val(), 0.0, 1.0, opt_.gpu.tol_flux), "wrong -pgpu_tol_flux");
    else if (s == "-pgpu_max_outer") PG_TRY(to_int(val(), 1, 100000000, opt_.gpu.max_outer), "wrong -pgpu_max_outer");
    else if (s == "-pgpu_max_inner") PG_TRY(to_int(val(), 1, 100000000, opt_.gpu.max_inner), "wrong -pgpu_max_inner");
    else if (s == "-pgpu_shift") PG_TRY(to_double(val(), 0.0, 10.0, opt_.gpu.shift), "wrong -pgpu_shift");
    else if (s == "-pgpu_device") PG_TRY(to_int(val(), 0, 1024, opt_.device), "wrong -pgpu_device");
    else if (s == "-pgpu_verbose") opt_.gpu.verbose = 1;
    else if (s == "-vtk" || s == "-petsc_dump") {
      // PETSc boolean options: the flag alone means on, or an explicit value follows
      bool on = true;
      if (a + 1 < argc) {
        const std::string v(argv[a + 1]);
        if (v == "1" || v == "true" || v == "yes") a++;
        else if (v == "0" || v == "false" || v == "no") on = false, a++;
      }
      (s == "-vtk" ? opt_.vtk : opt_.dump) = on;
    } else if (s == "-vtk_interval") PG_TRY(to_int(val(), 1, INT_MAX, opt_.vtk_interval), "wrong -vtk_interval");
    // other options (PETSc/SLEPc, -vtk, ...) are accepted and ignored
  }
  print("\nInitialize...");
  st_ = ParseState();
  PG_TRY(parse(filename, st_), "unable to parse " + filename);
  if (st_.vtk_set) {
    opt_.vtk = st_.vtk;
    opt_.vtk_interval = st_.vtk_interval;
  }
  if (st_.dump_set) opt_.dump = st_.dump;
  dt = st_.dt;
  // Driver::getMainSolver (Driver.cxx:115-129): the only solver, or the one named "main"
  PG_CHECK(st_.solvers.empty(), "no solvers defined");
  solver_ = nullptr;
  if (st_.solvers.size() == 1) {
    solver_ = st_.solvers[0].get();
  } else {
    for (auto& s : st_.solvers)
      if (s->name() == "main") solver_ = s.get();
    PG_CHECK(!solver_, "unable to find the main solver");
  }
  PG_TRY(solver_->initialize(*st_.mesh, st_.materials, opt_, !dt.empty()), "unable to initialize the solver");
  print("Done.");
  return 0;
}

int Driver::solve(int n, double dt, double t) {
  PG_CHECK(!solver_, "the driver is not initialized");
  print("\n--------------------------------");
  print(n == 0 ? "\nSolve steady state...\n" : "\nSolve time step " + std::to_string(n) + "...\n");
  auto t1 = std::chrono::steady_clock::now();
  PG_TRY(solver_->solve(n, dt, t), "unable to get the solution");
  auto t2 = std::chrono::steady_clock::now();
  if (opt_.verbose && !opt_.silent) {
    double s = std::chrono::duration<double>(t2 - t1).count();
    std::cout << std::scientific << std::setprecision(3) << "Solution time: " << s << "." << std::endl;
  }
  if (n > 0 && !opt_.silent)
    std::cout << std::scientific << std::setprecision(3) << "Time step size: " << dt << "." << std::endl
              << "Physical time: " << t << "." << std::endl;
  PG_TRY(solver_->output(n), "unable to output the solution");
  print("\nDone.");
  return 0;
}

int Driver::finalize() {
  print("\n--------------------------------");
  print("\nFinalize...");
  if (solver_) PG_TRY(solver_->finalize(), "unable to finalize the solver");
  solver_ = nullptr;
  st_ = ParseState();
  print("Done.\n");
  return 0;
}

}  // namespace pg

// ------------------------------------------------------------------------------------
// C API (pampa.cxx:5-115).  One global driver, not re-entrant, as in the reference.
// ------------------------------------------------------------------------------------

static pg::Driver g_pampa;

extern "C" {

void pampa_initialize(int argc, char* argv[], double** dt, int* ndt, int* error) {
  std::vector<double> dt0;
  *error = g_pampa.initialize(argc, argv, dt0);
  if (*error > 0) {
    std::printf("Error in pampa.initialize().\n");
    return;
  }
  *ndt = (int)dt0.size();
  *dt = new double[dt0.size() > 0 ? dt0.size() : 1];
  for (size_t i = 0; i < dt0.size(); i++) (*dt)[i] = dt0[i];
}

void pampa_initialize_steady_state(int argc, char* argv[], int* error) {
  std::vector<double> dt0;
  *error = g_pampa.initialize(argc, argv, dt0);
  if (*error > 0) std::printf("Error in pampa.initialize().\n");
}

void pampa_solve(int n, double dt, double t, int* error) {
  *error = g_pampa.solve(n, dt, t);
  if (*error > 0) std::printf("Error in pampa.solve().\n");
}

void pampa_solve_steady_state(int* error) {
  pampa_solve(0, 0.0, 0.0, error);
  if (*error > 0) std::printf("Error in pampa_solve().\n");
}

void pampa_finalize(double** dt, int* error) {
  *error = g_pampa.finalize();
  if (*error > 0) {
    std::printf("Error in pampa.finalize().\n");
    return;
  }
  delete[] *dt;
  *dt = nullptr;
}

void pampa_finalize_steady_state(int* error) {
  *error = g_pampa.finalize();
  if (*error > 0) std::printf("Error in pampa.finalize().\n");
}

void pampa_get_field(double* v, const char name[], int* error) {
  pg::Solver* s = g_pampa.solver();
  *error = s ? s->getField(v, std::string(name)) : 1;
  if (*error > 0) std::printf("Error in pampa.getField().\n");
}

void pampa_set_field(const double* v, const char name[], int* error) {
  pg::Solver* s = g_pampa.solver();
  *error = s ? s->setField(v, std::string(name)) : 1;
  if (*error > 0) std::printf("Error in pampa.setField().\n");
}

void pampa_get_keff(double* keff, int* error) {
  auto* s = g_pampa.solver() ? g_pampa.solver()->neutronic() : nullptr;
  *error = s ? 0 : 1;
  if (s) *keff = s->keff();
}

void pampa_get_field_size(const char name[], int* size, int* error) {
  pg::Solver* s = g_pampa.solver();
  *error = s ? s->fieldSize(std::string(name), *size) : 1;
}

void pampa_get_problem(pgpu_problem** problem, int* error) {
  auto* s = g_pampa.solver() ? g_pampa.solver()->neutronic() : nullptr;
  *error = s ? s->problem(problem) : 1;
  if (*error > 0) std::printf("Error in pampa_get_problem().\n");
}

void pampa_get_solve_stats(int* outer, int* inner, double* seconds, int* error) {
  auto* s = g_pampa.solver() ? g_pampa.solver()->neutronic() : nullptr;
  *error = s ? 0 : 1;
  if (!s) return;
  *outer = s->stats().outer_iterations;
  *inner = s->stats().inner_iterations;
  *seconds = s->stats().seconds;
}

}  // extern "C"
