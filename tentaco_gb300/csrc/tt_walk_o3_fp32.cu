// MTTKRP lean and staged walk kernels, order 3, storage fp32.
#define TT_ORDER 3
#define TT_PREC kFP32
#define TT_LOOKUP walk_launcher_o3_fp32
#define TT_LOOKUP_FLAT walk_launcher_o3_fp32_flat
#define TT_LOOKUP_TMA walk_launcher_o3_fp32_tma
#include "tt_walk_inst.cuh"
