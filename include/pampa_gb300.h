/*
 * pampa_gb300 -- GB300-native k-eigenvalue solver for pampa's neutronics hot path.
 *
 * Two C-ABI layers live in libpampa_gb300.so:
 *
 *   1. The drop-in driver API.  Same names, arguments and error convention as the
 *      reference's C API (src/pampa.hxx:5-27): `*error` is 0 on success and > 0 on
 *      failure, with a "file:line: error: message." line printed on stdout.  A
 *      program linked against the reference's libpampa.so relinks against this
 *      library unchanged; `.pmp` inputs are read as the reference reads them.
 *
 *   2. The GPU operator API (pgpu_*).  Plain pointers and sizes; every device buffer
 *      is owned by a pgpu problem handle and every host buffer by the caller.  The
 *      drop-in driver's DiffusionSolver / SNSolver classes call it; tests and
 *      benchmarks may call it directly.  Return value: PGPU_OK or a PGPU_ERR_* code,
 *      with pgpu_last_error() giving a message.  Iterations never spin forever: each
 *      loop has a cap and reports PGPU_ERR_NOT_CONVERGED when it runs out.
 *
 * Layouts follow the reference's global row numbering (NeutronicSolver.hxx:46 and
 * SNSolver.hxx:37-38): scalar flux phi[i*G + g], angular flux psi[(i*G + g)*M + m].
 * Face-indexed arrays are face-major with the cell index innermost: a[f*num_cells + i]
 * (a[f*num_cells*G + i*G + g] for per-group data) so that consecutive GPU threads
 * read consecutive addresses.
 */
#ifndef PAMPA_GB300_H
#define PAMPA_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------
 * 1. Drop-in driver API (replaces src/pampa.hxx:5-27 of the reference)
 * ---------------------------------------------------------------------------- */

/* Replaces pampa_initialize (pampa.hxx:8, pampa.cxx:11-36).  argv[1] is the .pmp
 * input; other arguments are options (-verbose, -silent, -pgpu_precision fp64|mixed,
 * -pgpu_tol_k X, -pgpu_tol_flux X, -pgpu_max_outer N, -pgpu_shift X, -pgpu_device N).  *dt receives a
 * new[]-allocated copy of the input's time steps, freed by pampa_finalize. */
void pampa_initialize(int argc, char* argv[], double** dt, int* ndt, int* error);

/* Replaces pampa_initialize_steady_state (pampa.hxx:11, pampa.cxx:39-57). */
void pampa_initialize_steady_state(int argc, char* argv[], int* error);

/* Replaces pampa_solve (pampa.hxx:14, pampa.cxx:60-66).  n = 0 is the steady-state
 * k-eigenvalue solve; n > 0 is a transient step of size dt (diffusion solvers; it needs
 * the steady state solved first and reports an error for SN solvers). */
void pampa_solve(int n, double dt, double t, int* error);

/* Replaces pampa_solve_steady_state (pampa.hxx:17, pampa.cxx:69-75). */
void pampa_solve_steady_state(int* error);

/* Replaces pampa_finalize (pampa.hxx:20, pampa.cxx:78-88). */
void pampa_finalize(double** dt, int* error);

/* Replaces pampa_finalize_steady_state (pampa.hxx:23, pampa.cxx:91-96). */
void pampa_finalize_steady_state(int* error);

/* Replaces pampa_get_field (pampa.hxx:26, pampa.cxx:99-105).  Field names as in the
 * reference: "scalar-flux", "angular-flux" (SN), "power", "production-rate",
 * "temperature", "delayed-source". */
void pampa_get_field(double* v, const char name[], int* error);

/* Replaces pampa_set_field (pampa.hxx:29, pampa.cxx:108-114). */
void pampa_set_field(const double* v, const char name[], int* error);

/* Additions beside the reference API (no counterpart there): the multiplication
 * factor printed by NeutronicSolver::printLog (NeutronicSolver.cxx:122), the size of a
 * field, and the statistics of the last solve. */
void pampa_get_keff(double* keff, int* error);
void pampa_get_field_size(const char name[], int* size, int* error);
void pampa_get_solve_stats(int* outer_iterations, int* inner_iterations, double* seconds,
                           int* error);

/* The device-resident problem behind the driver's solver, assembled and uploaded on first
 * use (no counterpart in the reference).  It stays owned by the driver: do not destroy it.
 * Lets callers reach the pgpu_* layer (e.g. pgpu_sn_apply) for an input read by the
 * drop-in parser. */
typedef struct pgpu_problem pgpu_problem;
void pampa_get_problem(pgpu_problem** problem, int* error);

/* ------------------------------------------------------------------------------
 * 2. GPU operator API
 * ---------------------------------------------------------------------------- */

enum {
  PGPU_OK = 0,
  PGPU_ERR_INVALID = 1,        /* bad argument or size                              */
  PGPU_ERR_CUDA = 2,           /* CUDA runtime error (message has the CUDA string)  */
  PGPU_ERR_NOT_CONVERGED = 3,  /* an iteration cap was reached                      */
  PGPU_ERR_NEGATIVE_FLUX = 4,  /* normalised flux has negative entries              */
  PGPU_ERR_NAN = 5,            /* a reduction produced NaN/Inf                       */
  PGPU_ERR_NO_MEMORY = 6,      /* device memory budget exceeded                     */
  PGPU_ERR_TIMEOUT = 7         /* a bounded device-side wait ran out; the kernel     */
                               /* returned early and the results are not valid       */
};

enum { PGPU_FP64 = 0, PGPU_MIXED = 1 };

/* pgpu_problem (declared above) is opaque: operator + iterates on one GPU. */

typedef struct {
  int precision;        /* PGPU_FP64 (default) or PGPU_MIXED (FP32 inner, FP64 outer)  */
  double tol_k;         /* |k_n - k_{n-1}| stop criterion            (default 1e-10)   */
  double tol_flux;      /* relative change of the fission source     (default 1e-9)    */
  int max_outer;        /* outer (eigen) iteration cap               (default 5000)    */
  int max_inner;        /* inner Krylov iteration cap per solve      (default 2000)    */
  double power;         /* normalisation target, NeutronicSolver.hxx:17 (default 1.0)  */
  int verbose;          /* print one line per outer iteration when > 0                 */
  int profile;          /* time the dominant kernel with CUDA events (default 0)       */
  double shift;         /* Wielandt shift once k has settled: the inner solves use     */
                        /* R - F / (k (1 + shift)); 0 = plain power iteration, < 0 =   */
                        /* the solver's default (0.02 diffusion, 0.05 SN; default -1)  */
} pgpu_options;

typedef struct {
  double keff;
  int outer_iterations;
  int inner_iterations;  /* total inner Krylov iterations                                */
  int sweeps;            /* SN only: transport sweeps                                    */
  double residual;       /* final relative eigen-residual estimate                       */
  double seconds;        /* device time of the solve (CUDA events)                       */
  int status;            /* PGPU_* code                                                  */
  long long launches;    /* kernels launched by the solve                                */
  /* Dominant kernel (transport sweep for SN, SpMV for diffusion), filled when
   * options.profile != 0: device seconds inside it (CUDA events on the launching
   * stream), its launches, and the algorithmic bytes those launches must move. */
  double kernel_seconds;
  long long kernel_launches;
  double kernel_bytes;
  char kernel_name[32];  /* name of that kernel (NUL-terminated)                         */
} pgpu_stats;

/* Fill *opt with the defaults listed above. */
void pgpu_default_options(pgpu_options* opt);

/* Message of the last error on the calling thread. */
const char* pgpu_last_error(void);

/* Multigroup diffusion operator R and fission operator F of DiffusionSolver::
 * buildMatrices (DiffusionSolver.cxx:88-320, n = 0), in cell-stencil form:
 *   R[(i,g),(i,g)]            = diag[i*G+g]
 *   R[(i,g),(i,g2)], g2 != g  = -sigma_s[mat(i)][g2][g] * volume[i]
 *   R[(i,g),(nbr,g)]          = offdiag[f*num_cells*G + i*G + g], nbr = neighbors[f*num_cells+i]
 *   F[(i,g),(i,g2)]           = chi[mat(i)][g] * nu_sigma_f[mat(i)][g2] * volume[i]
 * neighbors[] < 0 marks a boundary or absent face (its offdiag entry is ignored). */
typedef struct {
  int num_cells, num_groups, num_faces, num_materials;
  const int* neighbors;          /* [num_faces][num_cells]                        */
  const double* offdiag;         /* [num_faces][num_cells*G]                      */
  const double* diag;            /* [num_cells*G]                                 */
  const int* materials;          /* [num_cells], 0-based                          */
  const double* volumes;         /* [num_cells]                                   */
  const double* sigma_s;         /* [num_materials][G][G], [from][to]             */
  const double* chi;             /* [num_materials][G], effective spectrum        */
  const double* nu_sigma_f;      /* [num_materials][G]                            */
  const double* kappa_sigma_f;   /* [num_materials][G]                            */
} pgpu_diffusion_operator;

/* Upload a diffusion operator to `device` (HBM-resident until destroy). */
int pgpu_diffusion_create(int device, const pgpu_diffusion_operator* op, pgpu_problem** out);

/* Apply R to a host vector (y = R x, both num_cells*G).  Test hook for operator parity. */
int pgpu_diffusion_apply(pgpu_problem* p, const double* x, double* y);

/* SN boundary kinds per face (SNSolver.cxx:445-566). */
enum { PGPU_FACE_INTERIOR = 0, PGPU_FACE_VACUUM = 1, PGPU_FACE_REFLECTIVE = 2,
       PGPU_FACE_NONE = 3 };

/* Discrete-ordinates operator of SNSolver::buildMatrices (SNSolver.cxx:344-631, n = 0)
 * in matrix-free form.  Per face f of cell i (face-major arrays as above):
 *   face_kind[f*n+i]       PGPU_FACE_*
 *   neighbors[f*n+i]       neighbour cell (interior faces)
 *   areas[f*n+i], normals[(f*n+i)*3+d]
 *   gauss[(f*n+i)*4+c]     the four face-flux weights of SNSolver.cxx:192-199
 *   reflect_axis[f*n+i]    0/1/2: axis used to reflect directions at a reflective face
 *   ls_weight[(f*n+i)*F+f2] LS boundary correction dp_f . c_f2 (SNSolver.cxx:486-513);
 *                          only read for vacuum faces when use_ls != 0, may be NULL.
 * Quadrature: directions[m*3+d], weights[m], reflected[m*3+axis] (AngularQuadratureSet).
 * Materials as for diffusion (sigma_t is the total cross section). */
typedef struct {
  int num_cells, num_groups, num_dirs, num_faces, num_materials;
  int use_ls;
  const int* num_cell_faces;     /* [num_cells]                                   */
  const int* face_kind;
  const int* neighbors;
  const double* areas;
  const double* normals;
  const double* gauss;
  const int* reflect_axis;
  const double* ls_weight;
  const int* materials;
  const double* volumes;
  const double* directions;
  const double* weights;
  const int* reflected;
  const double* sigma_t;         /* [num_materials][G]                            */
  const double* sigma_s;         /* [num_materials][G][G]                         */
  const double* chi;
  const double* nu_sigma_f;
  const double* kappa_sigma_f;
  /* Optional: the mesh is a full nx*ny*nz Cartesian box in the reference's cell order
   * (x fastest, faces -y,+x,+y,-x,-z,+z).  Set all three to 0 otherwise.  When given and
   * verified, sweeps use tiles of 4x4x4 cells instead of per-cell upwind levels. */
  int cart_nx, cart_ny, cart_nz;
} pgpu_sn_operator;

/* Upload an SN operator; builds the per-direction upwind sweep schedule. */
int pgpu_sn_create(int device, const pgpu_sn_operator* op, pgpu_problem** out);

/* Apply the SN R to a host vector (num_cells*G*M).  Test hook for operator parity. */
int pgpu_sn_apply(pgpu_problem* p, const double* x, double* y);

/* Solve R x = (1/k) F x on the GPU, starting from a flat flux.  Results stay on the
 * device; read them with pgpu_problem_get_*.  Returns the solve status. */
int pgpu_problem_solve(pgpu_problem* p, const pgpu_options* opt, pgpu_stats* stats);

/* Linear solve with a diffusion problem's operator: (R - lam F) x = b, F[(i,g),(i,g2)] =
 * chi[mat(i)][g] nu_sigma_f[mat(i)][g2] V_i as in pgpu_diffusion_operator.  This is the
 * transient step of DiffusionSolver (DiffusionSolver.cxx:108-175 assembles R with the
 * 1/(v dt) terms on its diagonal and -(1 - beta) chi_p nu_sigma_f V / keff in-cell terms;
 * getSolution n > 0, :337-345, solves it with KSP, petsc.cxx:147-172): the caller
 * creates the problem with that diagonal and chi = (1 - beta) chi_prompt and passes
 * lam = 1/keff.  x (host, num_cells*G) is the initial guess on entry and the solution on
 * return; b is host memory.  Converged when ||b - (R - lam F) x|| <= tol_flux ||b||
 * (options.tol_flux, at least 1e-14); PGPU_ERR_NOT_CONVERGED after max_inner Krylov
 * iterations.  options.precision selects FP64 or FP32 corrections with FP64 residuals.
 * stats: outer_iterations = refinement steps, inner_iterations = Krylov iterations,
 * residual = final relative residual.  Diffusion problems only (PGPU_ERR_INVALID else). */
int pgpu_problem_solve_linear(pgpu_problem* p, double lam, const double* b, double* x,
                              const pgpu_options* opt, pgpu_stats* stats);

/* Results of the last solve, normalised as NeutronicSolver::normalizeScalarFlux and
 * SNSolver::normalizeAngularFlux do (sum phi*kappa_sigma_f*V = power).  Host buffers:
 * phi[num_cells*G], psi[num_cells*G*M] (SN only), q and P [num_cells]. */
int pgpu_problem_get_keff(pgpu_problem* p, double* keff);
int pgpu_problem_get_scalar_flux(pgpu_problem* p, double* phi);
int pgpu_problem_get_angular_flux(pgpu_problem* p, double* psi);
int pgpu_problem_get_power(pgpu_problem* p, double* q, double* P, double* total_power);

/* Device memory held by the problem, in bytes. */
long long pgpu_problem_device_bytes(pgpu_problem* p);

/* Size the problem's grids for `sms` streaming multiprocessors (0: the whole device), for
 * callers that run several solves on one device at once: each solve's small kernels then
 * leave room for the others' instead of the streams taking turns on a full device.  Results
 * depend on the share (reduction order), not on what else runs.  Diffusion solves only;
 * SN solves ignore it.  PGPU_ERR_INVALID for a null problem or sms < 0. */
int pgpu_problem_set_sm_share(pgpu_problem* p, int sms);

/* Bytes copied host-to-device when the problem was created (the operator). */
long long pgpu_problem_upload_bytes(pgpu_problem* p);

void pgpu_problem_destroy(pgpu_problem* p);

/* Flux normalisation and power fields that allocate nothing (no counterpart in the
 * reference; it is the normalisation its NeutronicSolver::normalizeScalarFlux and
 * calculatePowerAndProductionRate apply).  For callers that cannot call cudaMalloc --
 * their device memory belongs to another allocator, or they must not grow the device
 * footprint after start-up.  Every pointer is a caller-owned device buffer:
 *   in:  materials[n], volumes[n], kappa_sigma_f[nm*G], nu_sigma_f[nm*G], phi[n*G]
 *   out: phi_out[n*G] = phi * power / p0 with p0 = sum phi kappa_sigma_f V,
 *        q[n] (cell power), P[n] (production rate, divided by keff),
 *        total_power[1] and negatives[1] (may be NULL)
 * Work goes into `stream` (a cudaStream_t; NULL = legacy default stream of the current
 * device) and runs on the device that owns it; every buffer must live on that device.
 * Any group count is accepted.  The scratch is a fixed __device__ array inside the
 * library holding at most 1,048,576 cells; larger num_cells is rejected with
 * PGPU_ERR_INVALID before anything is queued.  The first call on a device looks up that
 * array's device address (cudaGetSymbolAddress) and must happen before any stream
 * capture.  All calls share the one array and it keeps the previous call's contents:
 * calls that overlap on the GPU (different streams, no ordering) race, so order them
 * on one stream or with events.  A flux whose power p0 is not positive and finite (an
 * all-zero flux, no fissile material, NaN) cannot be normalised: phi_out, q and P are
 * then set to zero, *total_power to 0 and *negatives to -1, which is the marker to check
 * after the stream has run (the return value only reports argument and launch errors). */
int pgpu_normalize_power_noalloc(int num_cells, int num_groups, const int* materials, const double* volumes,
                                 const double* kappa_sigma_f, const double* nu_sigma_f, const double* phi,
                                 double power, double keff, double* phi_out, double* q, double* P,
                                 double* total_power, int* negatives, void* stream);

/* ------------------------------------------------------------------------------
 * 4. Serving: continuous batching of independent k-eigenvalue solves on one GPU
 *    (new entry points beside the single-solve Solver path; the reference has no
 *    equivalent).  Requests are copied at submission and admitted first-in first-out
 *    as soon as one of `slots` workers is free and the request's device footprint fits
 *    in hbm_fraction of the device memory that was free at creation; each admitted
 *    request is uploaded, solved on its own stream and freed, so solves of different
 *    sizes overlap on the device.  A request larger than the whole budget is rejected
 *    with PGPU_ERR_NO_MEMORY.  Results do not depend on the other requests in flight.
 *    Submission, polling and waiting may come from any host thread.
 * ---------------------------------------------------------------------------- */
typedef struct pgpu_server pgpu_server;

int pgpu_serve_create(int device, int slots, double hbm_fraction, pgpu_server** out);
long long pgpu_serve_budget_bytes(pgpu_server* s);
/* SMs each solve started from now on sizes its grids for (pgpu_problem_set_sm_share);
 * the server's default is 3 / slots of the device (0, the whole device, for one slot). */
int pgpu_serve_set_sm_share(pgpu_server* s, int sms);
int pgpu_serve_submit_diffusion(pgpu_server* s, const pgpu_diffusion_operator* op, const pgpu_options* opt,
                                int want_flux, long long* id);
int pgpu_serve_submit_sn(pgpu_server* s, const pgpu_sn_operator* op, const pgpu_options* opt, int want_flux,
                         long long* id);
/* *done = 1 once the request's solve has finished (successfully or not). */
int pgpu_serve_poll(pgpu_server* s, long long id, int* done);
/* Blocks until the request is done and releases it; returns its solve status.  Outputs
 * may be NULL: stats, keff, phi (num_cells*G, only when submitted with want_flux) and
 * times[3] = {queueing, upload + solve + read-back, total latency} in seconds. */
int pgpu_serve_wait(pgpu_server* s, long long id, pgpu_stats* stats, double* keff, double* phi, double* times);
/* Finishes every submitted request, then stops the workers and frees the server. */
int pgpu_serve_destroy(pgpu_server* s);

#ifdef __cplusplus
}
#endif

#endif /* PAMPA_GB300_H */
