// Cooperative advance kernel, 32 lanes per cell, 16 warps per block.
#include "generated/coop_prog_g32.h"
#define WR_COOP_G 32
#define WR_COOP_W 16
#include "wr_adv_coop.cuh"
