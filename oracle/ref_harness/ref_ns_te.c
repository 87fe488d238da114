/* Oracle build only: compiles the reference's non-standard FDTD TE (nsFdtdTE.c) solver
 * unmodified and exposes its file-static state to the test harness. */
#include "nsFdtdTE.c"

void refh_nste_init(void) { init(); }
double complex *refh_nste_field(int which)
{
  switch (which) { case 0: return Ex; case 1: return Ey; case 2: return Hz; }
  return NULL;
}
double *refh_nste_eps(int which)
{
  switch (which) { case 0: return EPS_EX; case 1: return EPS_EY; case 2: return EPS_HZ; }
  return NULL;
}
