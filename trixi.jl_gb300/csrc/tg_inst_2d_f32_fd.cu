// Element kernels: 2D, float arithmetic, volume integral "fd".
#define TG_D 2
#define TG_REAL float
#define TG_VI 1
#define TG_SUFFIX 2d_f32_fd
#include "tg_inst.cuh"
