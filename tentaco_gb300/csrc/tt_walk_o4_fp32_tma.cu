// MTTKRP TMA-gather walk kernels, order 4, storage fp32.
#define TT_ORDER 4
#define TT_PREC kFP32
#define TT_TMA_UNIT
#define TT_LOOKUP walk_launcher_o4_fp32_tma
#include "tt_walk_inst.cuh"
