/* Oracle build only: compiles the reference's split-field TM (fdtdTM.c) solver
 * unmodified and exposes its file-static state to the test harness. */
#include "fdtdTM.c"

void refh_splittm_init(void) { init(); }
double complex *refh_splittm_field(int which)
{
  switch (which) { case 0: return Ez; case 1: return Hx; case 2: return Hy; }
  return NULL;
}
double *refh_splittm_eps(int which)
{
  switch (which) { case 0: return EPS_EZ; case 1: return EPS_HX; case 2: return EPS_HY; }
  return NULL;
}
