// Element kernels: 3D, double arithmetic, volume integral "hg".
#define TG_D 3
#define TG_REAL double
#define TG_VI 2
#define TG_SUFFIX 3d_f64_hg
#include "tg_inst.cuh"
