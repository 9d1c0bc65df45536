// Element kernels: 3D, float arithmetic, volume integral "weak".
#define TG_D 3
#define TG_REAL float
#define TG_VI 0
#define TG_SUFFIX 3d_f32_weak
#include "tg_inst.cuh"
