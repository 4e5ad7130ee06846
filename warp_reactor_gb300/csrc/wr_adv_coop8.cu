// Cooperative advance kernel, 8 lanes per cell (warps per block: generated/coop_prog_g8.h).
#include "generated/coop_prog_g8.h"
#define WR_COOP_G 8
#include "wr_adv_coop.cuh"
