// Mixed-precision element kernels: 2D, volume integral "fd".
#define TG_D 2
#define TG_VI 1
#define TG_SUFFIX 2d_fd
#include "tg_inst_mixed.cuh"
