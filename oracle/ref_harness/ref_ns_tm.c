/* Oracle build only: compiles the reference's non-standard FDTD TM (nsFdtdTM.c) solver
 * unmodified and exposes its file-static state to the test harness. */
#include "nsFdtdTM.c"

void refh_nstm_init(void) { init(); }
double complex *refh_nstm_field(int which)
{
  switch (which) { case 0: return Ez; case 1: return Hx; case 2: return Hy; }
  return NULL;
}
double *refh_nstm_eps(int which)
{
  switch (which) { case 0: return EPS_EZ; case 1: return EPS_HX; case 2: return EPS_HY; }
  return NULL;
}
