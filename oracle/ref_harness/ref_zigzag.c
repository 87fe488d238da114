/* Oracle build only: the reference's zigzagModel.c unmodified, plus a setter
 * for the structure its nextStructure() loop would otherwise walk through
 * (width, thickness, layer count, angle; zigzagModel.c:28-31). */
#include "zigzagModel.c"

void refh_zigzag_set(int width, int thick, int layers, int deg)
{
  width_nm = width;
  thickness_nm = thick;
  layerNum = layers;
  degree = deg;
}
