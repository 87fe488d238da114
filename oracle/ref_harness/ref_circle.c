/* Oracle build only: the reference's circleModel.c unmodified, plus setters for
 * its compile-time parameters (radius before init, permittivity after init). */
#include "circleModel.c"

void refh_circle_set_radius_nm(int r) { radius_nm = r; }
void refh_circle_set_eps(double e) { epsilon_s = e; }
double refh_circle_get_eps(void) { return epsilon_s; }
