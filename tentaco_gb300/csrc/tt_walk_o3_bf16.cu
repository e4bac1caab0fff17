// MTTKRP lean and staged walk kernels, order 3, storage bf16.
#define TT_ORDER 3
#define TT_PREC kBF16
#define TT_LOOKUP walk_launcher_o3_bf16
#define TT_LOOKUP_FLAT walk_launcher_o3_bf16_flat
#define TT_LOOKUP_TMA walk_launcher_o3_bf16_tma
#include "tt_walk_inst.cuh"
