/* Oracle build only: compiles the reference's MPI TM UPML solver unmodified
 * (mpiTM_UPML.c) and exposes its file-static state to the test harness. */
#include "mpiTM_UPML.c"

void refh_mpitm_init(void) { init(); }
void refh_mpitm_dims(int *spx, int *spy) { *spx = SUB_N_PX; *spy = SUB_N_PY; }
double complex *refh_mpitm_field(int which)
{
  switch (which) {
  case 0: return Ez; case 1: return Hx; case 2: return Hy;
  case 3: return Jz; case 4: return Dz; case 5: return Mx;
  case 6: return Bx; case 7: return My; case 8: return By;
  }
  return NULL;
}
double *refh_mpitm_eps(int which)
{
  switch (which) { case 0: return EPS_EZ; case 1: return EPS_HX; case 2: return EPS_HY; }
  return NULL;
}
double complex *refh_mpitm_ntff(int which)
{
  switch (which) { case 0: return Ux; case 1: return Uy; case 2: return Wz; }
  return NULL;
}
