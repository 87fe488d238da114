/* Oracle build only: compiles the reference's serial TM UPML solver unmodified
 * (fdtdTM_upml.c) and exposes its file-static state to the test harness. */
#include "fdtdTM_upml.c"

void refh_sertm_init(void) { init(); }
double complex *refh_sertm_field(int which)
{
  switch (which) { case 0: return Ez; case 1: return Hx; case 2: return Hy; }
  return NULL;
}
double *refh_sertm_eps(int which)
{
  switch (which) { case 0: return EPS_EZ; case 1: return EPS_HX; case 2: return EPS_HY; }
  return NULL;
}
double complex *refh_sertm_ntff(int which)
{
  switch (which) { case 0: return Ux; case 1: return Uy; case 2: return Wz; }
  return NULL;
}
/* ntffTM_TimeOutput writes "<angle>[deg].txt" and the binary spectrum into cwd. */
void refh_sertm_time_output(void) { ntffTM_TimeOutput(Ux, Uy, Wz); }
