// MTTKRP strip walk kernels, order 3, storage bf16.
#define TT_ORDER 3
#define TT_PREC kBF16
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o3_bf16_strip
#include "tt_walk_inst.cuh"
