/* Oracle build only: compiles the reference's serial TE UPML solver unmodified
 * (fdtdTE_upml.c) and exposes its file-static state to the test harness. */
#include "fdtdTE_upml.c"

void refh_serte_init(void) { init(); }
double complex *refh_serte_field(int which)
{
  switch (which) { case 0: return Ex; case 1: return Ey; case 2: return Hz; }
  return NULL;
}
double *refh_serte_eps(int which)
{
  switch (which) { case 0: return EPS_EX; case 1: return EPS_EY; case 2: return EPS_HZ; }
  return NULL;
}
double complex *refh_serte_ntff(int which)
{
  switch (which) { case 0: return Wx; case 1: return Wy; case 2: return Uz; }
  return NULL;
}
void refh_serte_time_output(void) { ntffTE_TimeOutput(Wx, Wy, Uz); }
