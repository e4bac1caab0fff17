// MTTKRP strip walk kernels, order 4, storage bf16f.
#define TT_ORDER 4
#define TT_PREC kBF16F
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o4_bf16f_strip
#include "tt_walk_inst.cuh"
