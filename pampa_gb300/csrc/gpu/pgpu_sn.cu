// Discrete-ordinates k-eigenvalue solve on one GPU (placeholder until the sweep lands).
#include "pgpu_internal.cuh"

namespace pgpu {
struct SNData {};
int sn_solve(pgpu_problem*, const pgpu_options*, pgpu_stats*) { return fail(PGPU_ERR_INVALID, "SN not built"); }
int sn_get_flux(pgpu_problem*, double*) { return fail(PGPU_ERR_INVALID, "SN not built"); }
int sn_get_angular(pgpu_problem*, double*) { return fail(PGPU_ERR_INVALID, "SN not built"); }
int sn_get_power(pgpu_problem*, double*, double*, double*) { return fail(PGPU_ERR_INVALID, "SN not built"); }
void sn_destroy(pgpu_problem* p) { delete p->sn; p->sn = nullptr; }
}  // namespace pgpu

extern "C" {
int pgpu_sn_create(int, const pgpu_sn_operator*, pgpu_problem** out) { *out = nullptr; return pgpu::fail(PGPU_ERR_INVALID, "SN not built"); }
int pgpu_sn_apply(pgpu_problem*, const double*, double*) { return pgpu::fail(PGPU_ERR_INVALID, "SN not built"); }
}
