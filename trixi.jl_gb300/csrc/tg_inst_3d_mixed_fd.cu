// Mixed-precision element kernels: 3D, volume integral "fd".
#define TG_D 3
#define TG_VI 1
#define TG_SUFFIX 3d_fd
#include "tg_inst_mixed.cuh"
