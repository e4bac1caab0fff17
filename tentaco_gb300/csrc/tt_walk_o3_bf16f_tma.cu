// MTTKRP TMA-gather walk kernels, order 3, storage bf16f.
#define TT_ORDER 3
#define TT_PREC kBF16F
#define TT_TMA_UNIT
#define TT_LOOKUP walk_launcher_o3_bf16f_tma
#include "tt_walk_inst.cuh"
