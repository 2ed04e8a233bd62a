/*
 * CPU restatement of the upwind transport sweep -- TEST/BASELINE INFRASTRUCTURE ONLY.
 *
 * Used by bench.py's CPU legs (cpu_baseline, --impl reference) to time the sweep-based
 * k-eigenvalue solve on the host cores; tests may use it as a checker.  The product
 * never links it.
 *
 * It solves, cell by cell in upwind order, the rows of the reference's SN operator
 * (SNSolver.cxx:344-631) for pure upwind face interpolation (mixed-face-interpolation
 * 1.0) without the LS boundary correction:
 *   psi[i,g,m] * (sigma_t V + sum_{f: mu>0} w_i mu A)
 *       = q[i,g] - sum_{f: mu<0} w_j mu A psi[j,g,m] - sum_{reflective f: mu<0} mu A psi_in
 * with mu = Omega_m . n_f.  Levels come from the caller (cells of one level are mutually
 * independent for every direction of a pattern) and each level is split over OpenMP
 * threads.  moment() forms phi0[i,g] = sum_m w_m psi[i,g,m].
 *
 * Build: gcc -O3 -fopenmp -shared -fPIC cpu_sweep.c -o _ref/libcpu_sweep.so
 */
#include <stddef.h>

#ifdef _OPENMP
#include <omp.h>
#endif

enum { INTERIOR = 0, VACUUM = 1, REFLECTIVE = 2 };

int cpu_sweep_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void cpu_sweep(int n, int G, int M, int F, const int* nf, const int* kind, const int* nbr,
               const double* area, const double* nrm, const double* gauss, const int* rslot,
               const int* mat, const double* vol, const double* dirs, const double* st, int npat,
               const int* pat_dirs_ptr, const int* pat_dirs, const int* pat_lev_ptr,
               const int* pat_nlev, const int* lev_ptr, const int* order, const double* q,
               const double* bnd, double* psi, int nthreads) {
  int nlev = 0;
  for (int p = 0; p < npat; p++)
    if (pat_nlev[p] > nlev) nlev = pat_nlev[p];
  (void)F;
  for (int L = 0; L < nlev; L++) {
    for (int p = 0; p < npat; p++) {
      if (L >= pat_nlev[p]) continue;
      const int d0 = pat_dirs_ptr[p], nd = pat_dirs_ptr[p + 1] - d0;
      const int* lp = lev_ptr + pat_lev_ptr[p];
      const int c0 = lp[L], nc = lp[L + 1] - c0;
      const int* ord = order + (size_t)p * n;
      const long long items = (long long)nc * nd * G;
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (long long it = 0; it < items; it++) {
        const int di = (int)(it % nd);
        const long long rest = it / nd;
        const int g = (int)(rest % G);
        const int i = ord[c0 + (int)(rest / G)];
        const int m = pat_dirs[d0 + di];
        const double* om = dirs + (size_t)m * 3;
        double den = st[(size_t)mat[i] * G + g] * vol[i];
        double num = q[(size_t)i * G + g];
        for (int f = 0; f < nf[i]; f++) {
          const size_t o = (size_t)f * n + i;
          const double* nv = nrm + o * 3;
          const double mu = om[0] * nv[0] + om[1] * nv[1] + om[2] * nv[2];
          const double muA = mu * area[o];
          if (kind[o] == INTERIOR) {
            if (mu > 0.0) den += gauss[o * 4 + 0] * muA;
            else num -= gauss[o * 4 + 3] * muA * psi[((size_t)nbr[o] * G + g) * M + m];
          } else if (kind[o] == VACUUM) {
            if (mu > 0.0) den += muA;
          } else if (kind[o] == REFLECTIVE) {
            if (mu > 0.0) den += muA;
            else if (bnd) num -= muA * bnd[((size_t)rslot[o] * G + g) * M + m];
          }
        }
        psi[((size_t)i * G + g) * M + m] = num / den;
      }
    }
  }
}

void cpu_moment(long long rows, int M, const double* w, const double* psi, double* phi0, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (long long r = 0; r < rows; r++) {
    double s = 0.0;
    for (int m = 0; m < M; m++) s += w[m] * psi[r * M + m];
    phi0[r] = s;
  }
}
