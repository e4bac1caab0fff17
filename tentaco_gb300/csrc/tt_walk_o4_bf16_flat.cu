// MTTKRP flat walk kernels, order 4, storage bf16.
#define TT_ORDER 4
#define TT_PREC kBF16
#define TT_FLAT_UNIT
#define TT_LOOKUP walk_launcher_o4_bf16_flat
#include "tt_walk_inst.cuh"
