/* Oracle build only: compiles the reference's split-field TE (fdtdTE.c) solver
 * unmodified and exposes its file-static state to the test harness. */
#include "fdtdTE.c"

void refh_splitte_init(void) { init(); }
double complex *refh_splitte_field(int which)
{
  switch (which) { case 0: return Ex; case 1: return Ey; case 2: return Hz; }
  return NULL;
}
double *refh_splitte_eps(int which)
{
  switch (which) { case 0: return EPS_EX; case 1: return EPS_EY; case 2: return EPS_HZ; }
  return NULL;
}
