// Cooperative advance kernel, 8 lanes per cell, 6 warps per block.
#include "generated/coop_prog_g8.h"
#define WR_COOP_G 8
#define WR_COOP_W 6
#include "wr_adv_coop.cuh"
