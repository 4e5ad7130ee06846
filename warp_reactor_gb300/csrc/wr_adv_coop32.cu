// Cooperative advance kernel, 32 lanes per cell (warps per block: generated/coop_prog_g32.h).
#include "generated/coop_prog_g32.h"
#define WR_COOP_G 32
#include "wr_adv_coop.cuh"
