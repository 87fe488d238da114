// surrogate_ops.cu -- element-wise kernels of the far-field surrogate
// (filled in with the model).
#include <cuda_runtime.h>
