/*
 * CPU restatement of the upwind transport sweep -- TEST/BASELINE INFRASTRUCTURE ONLY.
 *
 * Used by oracle/sn_cpu.py, the CPU k-eigenvalue solve of the pure-upwind SN problem that
 * bench.py times as the CPU reference and that tests and the bench use as a checker at
 * sizes the oracle's direct solve cannot reach.  The product never links it.
 *
 * It solves, cell by cell in upwind order, the rows of the reference's SN operator
 * (SNSolver.cxx:344-631) for pure upwind face interpolation (mixed-face-interpolation
 * 1.0) without the LS boundary correction:
 *   psi[i,g,m] * (sigma_t V + sum_{f: mu>0} w_i mu A)
 *       = q[i,g] - sum_{f: mu<0} w_j mu A psi[j,g,m] - sum_{reflective f: mu<0} mu A psi_in
 * with mu = Omega_m . n_f and (w_i, w_j) the Gauss weights c0, c3 of SNSolver.cxx:192-199.
 * With the source isotropic, every (group, direction) pair is an independent sweep of the
 * mesh, so threads take whole sweeps of one group and one upwind pattern (angle-parallel,
 * no barrier inside a sweep).
 *
 * Build: gcc -O3 -fopenmp -shared -fPIC cpu_sweep.c -o _ref/libcpu_sweep.so
 */
#include <stdlib.h>
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

/* Upwind order of the cells for direction `om` (3 doubles): Kahn's algorithm over the
 * edges j -> i for every interior face of i with mu = om . n < 0 (j its neighbour),
 * always taking the smallest ready cell index, so that cells numbered row by row are
 * swept nearly in memory order.  Returns 0, or 1 when the graph has a cycle. */
int cpu_upwind_order(int n, int F, const int* nf, const int* kind, const int* nbr, const double* nrm,
                     const double* om, int* order) {
  int* indeg = (int*)calloc((size_t)n, sizeof(int));
  int* head = (int*)calloc((size_t)n + 1, sizeof(int));
  int* heap = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int rc = 0;
  (void)F;
  for (int i = 0; i < n; i++)
    for (int f = 0; f < nf[i]; f++) {
      const size_t o = (size_t)f * n + i;
      const double* nv = nrm + o * 3;
      if (kind[o] == INTERIOR && om[0] * nv[0] + om[1] * nv[1] + om[2] * nv[2] < 0.0) {
        head[nbr[o] + 1]++;
        indeg[i]++;
      }
    }
  for (int i = 0; i < n; i++) head[i + 1] += head[i];
  int* adj = (int*)malloc(sizeof(int) * (size_t)(head[n] > 0 ? head[n] : 1));
  int* fill = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++) fill[i] = head[i];
  for (int i = 0; i < n; i++)
    for (int f = 0; f < nf[i]; f++) {
      const size_t o = (size_t)f * n + i;
      const double* nv = nrm + o * 3;
      if (kind[o] == INTERIOR && om[0] * nv[0] + om[1] * nv[1] + om[2] * nv[2] < 0.0) adj[fill[nbr[o]]++] = i;
    }
  int hn = 0, cnt = 0;
  for (int i = 0; i < n; i++)
    if (indeg[i] == 0) heap[hn++] = i; /* increasing indices: already a min-heap */
  while (hn > 0) {
    const int top = heap[0];
    order[cnt++] = top;
    /* pop */
    int last = heap[--hn], k = 0;
    while (1) {
      int c = 2 * k + 1;
      if (c >= hn) break;
      if (c + 1 < hn && heap[c + 1] < heap[c]) c++;
      if (heap[c] >= last) break;
      heap[k] = heap[c];
      k = c;
    }
    if (hn > 0) heap[k] = last;
    /* release the downwind cells */
    for (int e = head[top]; e < head[top + 1]; e++) {
      const int j = adj[e];
      if (--indeg[j] == 0) {
        int c = hn++;
        while (c > 0 && heap[(c - 1) / 2] > j) {
          heap[c] = heap[(c - 1) / 2];
          c = (c - 1) / 2;
        }
        heap[c] = j;
      }
    }
  }
  if (cnt != n) rc = 1;
  free(indeg);
  free(head);
  free(heap);
  free(adj);
  free(fill);
  return rc;
}

/* One transport sweep of every group and direction.  A thread takes one (group, pattern)
 * at a time and walks the pattern's upwind cell order, updating the pattern's nd
 * directions of a cell together.  Storage is per (group, pattern) block b = g*npat + p,
 * each holding its directions contiguously per cell, so no two threads write the same
 * cache line and the direction loops vectorise:
 *   psi[pbase[b] + i*nd + d]                          angular flux
 *   tab[tbase[p] + ((c*G + g)*(1 + F) + k)*nd + d]     per cell class c: k = 0 the reciprocal
 *       diagonal rd, k = 1 + f the inflow coefficient a_f = -(mu_f w_in,f) rd of face f
 *       (0 on outflow, vacuum and absent faces), so psi = rd q + sum_f a_f psi_in,f
 *   bnd[bbase[b] + slot*nd + d]                       inflow at reflective face slots
 * upw[i*F + f] is the upwind neighbour of an interior face, -(slot + 2) for a reflective
 * face, -1 otherwise; fmask[p*ncls + c] has bit f set when face f of class c has a
 * non-zero coefficient for some direction of pattern p; q is the isotropic source [n*G]. */
/* The sweep of one (group, pattern) block over its cells, with the pattern's direction
 * count ND known at compile time (S2/S4/S6/S8 octants) or given at run time (ND = 0). */
#define SWEEP_BLOCK(ND)                                                                      \
  static void sweep_block_##ND(int n, int G, int F, int g, int nd_rt, int mask_stride,       \
                               const int* fmask, const int* ord, const int* upw,             \
                               const int* cls, const double* TP, const double* q,            \
                               const double* B, double* P) {                                 \
    const int nd = (ND) > 0 ? (ND) : nd_rt;                                                   \
    double v[(ND) > 0 ? (ND) : 256];                                                          \
    for (int k = 0; k < n; k++) {                                                             \
      const int i = ord[k];                                                                   \
      const int* u = upw + (size_t)i * F;                                                     \
      const double qi = q[(size_t)i * G + g];                                                 \
      const int c = cls[i];                                                                   \
      const int mask = fmask[c];                                                              \
      const double* T0 = TP + ((size_t)c * G + g) * (size_t)(1 + F) * nd;                    \
      for (int d = 0; d < nd; d++) v[d] = T0[d] * qi;                                         \
      for (int f = 0; f < F; f++) {                                                           \
        if (!((mask >> f) & 1)) continue;                                                     \
        const int j = u[f];                                                                   \
        if (j == -1) continue;                                                                \
        const double* src = j >= 0 ? P + (size_t)j * nd : (B ? B + (size_t)(-j - 2) * nd : 0); \
        if (!src) continue;                                                                   \
        const double* a = T0 + (size_t)(1 + f) * nd;                                          \
        for (int d = 0; d < nd; d++) v[d] += a[d] * src[d];                                   \
      }                                                                                       \
      double* out = P + (size_t)i * nd;                                                       \
      for (int d = 0; d < nd; d++) out[d] = v[d];                                             \
    }                                                                                         \
    (void)mask_stride;                                                                        \
  }
SWEEP_BLOCK(0)
SWEEP_BLOCK(1)
SWEEP_BLOCK(3)
SWEEP_BLOCK(6)
SWEEP_BLOCK(10)

void cpu_sweep_pat(int n, int G, int F, int npat, int ncls, const int* pat_nd, const long long* pbase,
                   const long long* tbase, const long long* bbase, const int* upw, const int* cls,
                   const int* fmask, const double* tab, const int* order, const double* q, const double* bnd,
                   double* psi, int nthreads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int task = 0; task < G * npat; task++) {
    const int g = task / npat, p = task - g * npat;
    const int nd = pat_nd[p];
    const int* ord = order + (size_t)p * n;
    const int* fm = fmask + (size_t)p * ncls;
    double* P = psi + pbase[task];
    const double* B = bnd ? bnd + bbase[task] : 0;
    const double* TP = tab + tbase[p];
    switch (nd) {
      case 1: sweep_block_1(n, G, F, g, nd, ncls, fm, ord, upw, cls, TP, q, B, P); break;
      case 3: sweep_block_3(n, G, F, g, nd, ncls, fm, ord, upw, cls, TP, q, B, P); break;
      case 6: sweep_block_6(n, G, F, g, nd, ncls, fm, ord, upw, cls, TP, q, B, P); break;
      case 10: sweep_block_10(n, G, F, g, nd, ncls, fm, ord, upw, cls, TP, q, B, P); break;
      default: sweep_block_0(n, G, F, g, nd, ncls, fm, ord, upw, cls, TP, q, B, P); break;
    }
  }
}

/* phi0[i*G + g] = sum over patterns p and their directions d of w[p][d] psi (layout above) */
void cpu_moment_pat(int n, int G, int npat, const int* pat_nd, const long long* pbase, const double* wpat,
                    const double* psi, double* phi0, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int i = 0; i < n; i++)
    for (int g = 0; g < G; g++) {
      double s = 0.0;
      const double* w = wpat;
      for (int p = 0; p < npat; p++) {
        const int nd = pat_nd[p];
        const double* ps = psi + pbase[g * npat + p] + (size_t)i * nd;
        for (int d = 0; d < nd; d++) s += w[d] * ps[d];
        w += nd;
      }
      phi0[(size_t)i * G + g] = s;
    }
}

/* Isotropic source q[i*G + g] = V_i sum_g2 (ss[mat][g2][g] + lam chi[mat][g] nsf[mat][g2]) phi0[i*G + g2]
 * (+ b[i*G + g] when b is not NULL). */
void cpu_source(int n, int G, const int* mat, const double* vol, const double* ss, const double* chi,
                const double* nsf, double lam, const double* phi0, const double* b, double* q, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int i = 0; i < n; i++) {
    const int mt = mat[i];
    const double* ph = phi0 + (size_t)i * G;
    const double* S = ss + (size_t)mt * G * G;
    double f = 0.0;
    if (lam != 0.0)
      for (int g2 = 0; g2 < G; g2++) f += nsf[(size_t)mt * G + g2] * ph[g2];
    for (int g = 0; g < G; g++) {
      double s = 0.0;
      for (int g2 = 0; g2 < G; g2++) s += S[g2 * G + g] * ph[g2];
      if (lam != 0.0) s += lam * chi[(size_t)mt * G + g] * f;
      s *= vol[i];
      q[(size_t)i * G + g] = b ? s + b[(size_t)i * G + g] : s;
    }
  }
}

/* h[k] = <V_k, w> for k < nv (V row-major [nv][L]) */
void cpu_dots(long long L, int nv, const double* V, const double* w, double* h, int nthreads) {
  for (int k = 0; k < nv; k++) h[k] = 0.0;
#pragma omp parallel num_threads(nthreads)
  {
    double part[64];
    for (int k = 0; k < nv; k++) part[k] = 0.0;
#pragma omp for schedule(static)
    for (long long l = 0; l < L; l++) {
      const double x = w[l];
      for (int k = 0; k < nv; k++) part[k] += V[(size_t)k * L + l] * x;
    }
#pragma omp critical
    for (int k = 0; k < nv; k++) h[k] += part[k];
  }
}

/* w -= sum_k h[k] V_k; returns ||w|| */
double cpu_sub_norm(long long L, int nv, const double* V, const double* h, double* w, int nthreads) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(nthreads)
  for (long long l = 0; l < L; l++) {
    double x = w[l];
    for (int k = 0; k < nv; k++) x -= h[k] * V[(size_t)k * L + l];
    w[l] = x;
    s += x * x;
  }
  return __builtin_sqrt(s);
}

double cpu_norm(long long L, const double* x, int nthreads) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(nthreads)
  for (long long l = 0; l < L; l++) s += x[l] * x[l];
  return __builtin_sqrt(s);
}
