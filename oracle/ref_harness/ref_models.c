/* Oracle build only: compiles the reference's model dispatch (models.c)
 * unmodified and lets the harness install its own epsilon callback, so golden
 * vectors can be made for arbitrary seeded permittivity maps. */
#include "models.c"

void refh_models_set_callback(double (*fn)(double, double, int, int))
{
  epsMethod = fn;
  initModelMethod = noModel_init;
  needSizeMethod = noModel_needSize;
  isFinishMethod = noModel_isFinish;
}
