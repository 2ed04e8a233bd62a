/*
 * A C front end of the drop-in API, for the tests.  It drives a calculation the way the
 * reference's C front end does (src/c/main.c:6-34): pampa_initialize with the command
 * line, pampa_solve for the steady state (n = 0) and then every time step of the input
 * with t accumulated from the returned dt list, and pampa_finalize; it exits with 1 after
 * printing a line when a call reports an error.  Built against include/pampa_gb300.h and
 * linked with libpampa_gb300.so.
 */
#include <stdio.h>

#include "pampa_gb300.h"

int main(int argc, char* argv[]) {
  int error = 0, ndt = 0;
  double* dt = NULL;
  pampa_initialize(argc, argv, &dt, &ndt, &error);
  if (error > 0) {
    printf("Error in pampa_initialize().\n");
    return 1;
  }
  double t = 0.0;
  for (int n = 0; n <= ndt; n++) {
    const double step = n > 0 ? dt[n - 1] : 0.0;
    t += step;
    pampa_solve(n, step, t, &error);
    if (error > 0) {
      printf("Error in pampa_solve().\n");
      return 1;
    }
  }
  pampa_finalize(&dt, &error);
  if (error > 0) {
    printf("Error in pampa_finalize().\n");
    return 1;
  }
  return 0;
}
