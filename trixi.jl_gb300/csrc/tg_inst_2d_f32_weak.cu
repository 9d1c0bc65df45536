// Element kernels: 2D, float arithmetic, volume integral "weak".
#define TG_D 2
#define TG_REAL float
#define TG_VI 0
#define TG_SUFFIX 2d_f32_weak
#include "tg_inst.cuh"
