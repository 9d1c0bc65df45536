// Element kernels: 2D, double arithmetic, volume integral "hg".
#define TG_D 2
#define TG_REAL double
#define TG_VI 2
#define TG_SUFFIX 2d_f64_hg
#include "tg_inst.cuh"
