// MTTKRP lean and staged walk kernels, order 4, storage bf16f.
#define TT_ORDER 4
#define TT_PREC kBF16F
#define TT_LOOKUP walk_launcher_o4_bf16f
#define TT_LOOKUP_FLAT walk_launcher_o4_bf16f_flat
#define TT_LOOKUP_TMA walk_launcher_o4_bf16f_tma
#include "tt_walk_inst.cuh"
