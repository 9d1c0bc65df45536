// Element kernels: 3D, double arithmetic, volume integral "weak".
#define TG_D 3
#define TG_REAL double
#define TG_VI 0
#define TG_SUFFIX 3d_f64_weak
#include "tg_inst.cuh"
