// MTTKRP strip walk kernels, order 4, storage bf16.
#define TT_ORDER 4
#define TT_PREC kBF16
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o4_bf16_strip
#include "tt_walk_inst.cuh"
