// kernels_f32c.cu -- the FP32c instantiations of the single-run step
// kernels and their launchers (kernels.cu, part 2).
#define QGW_KERNELS_PART 2
#include "kernels.cu"
