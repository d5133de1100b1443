// kernels_ens_f32c.cu -- the FP32c instantiations of the ensemble step
// kernels and their launchers (kernels_ens.cu, part 2).
#define QGW_ENS_PART 2
#include "kernels_ens.cu"
