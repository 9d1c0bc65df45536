// Mixed-precision element kernels: 3D, volume integral "hg".
#define TG_D 3
#define TG_VI 2
#define TG_SUFFIX 3d_hg
#include "tg_inst_mixed.cuh"
