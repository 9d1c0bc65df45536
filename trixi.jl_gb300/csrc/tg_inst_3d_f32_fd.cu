// Element kernels: 3D, float arithmetic, volume integral "fd".
#define TG_D 3
#define TG_REAL float
#define TG_VI 1
#define TG_SUFFIX 3d_f32_fd
#include "tg_inst.cuh"
