// Mixed-precision element kernels: 3D, volume integral "weak".
#define TG_D 3
#define TG_VI 0
#define TG_SUFFIX 3d_weak
#include "tg_inst_mixed.cuh"
