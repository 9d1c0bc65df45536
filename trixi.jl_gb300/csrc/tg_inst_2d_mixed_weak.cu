// Mixed-precision element kernels: 2D, volume integral "weak".
#define TG_D 2
#define TG_VI 0
#define TG_SUFFIX 2d_weak
#include "tg_inst_mixed.cuh"
