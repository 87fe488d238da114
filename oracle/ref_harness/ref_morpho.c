/* Oracle build only: the reference's morphoScaleModel.c unmodified, plus
 * setters for the structure parameters that the reference sweeps. */
#include "morphoScaleModel.c"

void refh_morpho_set(int width, int thick0, int thick1, int layers, int branch, double edge_rate)
{
  width_nm = width;
  thickness_nm[0] = thick0;
  thickness_nm[1] = thick1;
  layerNum = layers;
  branch_width_nm = branch;
  edge_width_rate = edge_rate;
}
void refh_morpho_set_eps(double e) { ep_s = e; }
