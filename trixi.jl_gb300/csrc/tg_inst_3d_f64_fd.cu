// Element kernels: 3D, double arithmetic, volume integral "fd".
#define TG_D 3
#define TG_REAL double
#define TG_VI 1
#define TG_SUFFIX 3d_f64_fd
#include "tg_inst.cuh"
