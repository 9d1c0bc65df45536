// Element kernels: 2D, double arithmetic, volume integral "weak".
#define TG_D 2
#define TG_REAL double
#define TG_VI 0
#define TG_SUFFIX 2d_f64_weak
#include "tg_inst.cuh"
