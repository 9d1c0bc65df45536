// Element kernels: 2D, float arithmetic, volume integral "hg".
#define TG_D 2
#define TG_REAL float
#define TG_VI 2
#define TG_SUFFIX 2d_f32_hg
#include "tg_inst.cuh"
