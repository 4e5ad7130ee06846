// Cooperative advance kernel, 16 lanes per cell (warps per block: generated/coop_prog_g16.h).
#include "generated/coop_prog_g16.h"
#define WR_COOP_G 16
#include "wr_adv_coop.cuh"
