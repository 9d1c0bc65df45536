// Mixed-precision element kernels: 2D, volume integral "hg".
#define TG_D 2
#define TG_VI 2
#define TG_SUFFIX 2d_hg
#include "tg_inst_mixed.cuh"
