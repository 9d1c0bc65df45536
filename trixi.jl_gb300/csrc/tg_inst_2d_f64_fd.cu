// Element kernels: 2D, double arithmetic, volume integral "fd".
#define TG_D 2
#define TG_REAL double
#define TG_VI 1
#define TG_SUFFIX 2d_f64_fd
#include "tg_inst.cuh"
