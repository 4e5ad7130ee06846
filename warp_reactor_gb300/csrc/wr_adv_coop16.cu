// Cooperative advance kernel, 16 lanes per cell, 12 warps per block.
#include "generated/coop_prog_g16.h"
#define WR_COOP_G 16
#define WR_COOP_W 12
#include "wr_adv_coop.cuh"
