// MTTKRP strip walk kernels, order 5, storage fp32.
#define TT_ORDER 5
#define TT_PREC kFP32
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o5_fp32_strip
#include "tt_walk_inst.cuh"
