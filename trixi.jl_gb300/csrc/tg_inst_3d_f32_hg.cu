// Element kernels: 3D, float arithmetic, volume integral "hg".
#define TG_D 3
#define TG_REAL float
#define TG_VI 2
#define TG_SUFFIX 3d_f32_hg
#include "tg_inst.cuh"
