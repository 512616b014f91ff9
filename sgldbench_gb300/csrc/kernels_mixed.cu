// Mixed-precision preconditioner kernels (FP32 V-cycle).  Filled in with the
// mixed solve path.
#include "sgld_internal.cuh"
