/* Oracle build only: compiles the reference's MPI TE UPML solver unmodified
 * (mpiTE_UPML.c) and exposes its file-static state to the test harness. */
#include "mpiTE_UPML.c"

void refh_mpite_init(void) { init(); }
void refh_mpite_dims(int *spx, int *spy) { *spx = SUB_N_PX; *spy = SUB_N_PY; }
double complex *refh_mpite_field(int which)
{
  switch (which) {
  case 0: return Ex; case 1: return Ey; case 2: return Hz;
  case 3: return Jx; case 4: return Dx; case 5: return Jy;
  case 6: return Dy; case 7: return Mz; case 8: return Bz;
  }
  return NULL;
}
double *refh_mpite_eps(int which)
{
  switch (which) { case 0: return EPS_EX; case 1: return EPS_EY; case 2: return EPS_HZ; }
  return NULL;
}
double complex *refh_mpite_ntff(int which)
{
  switch (which) { case 0: return Wx; case 1: return Wy; case 2: return Uz; }
  return NULL;
}
