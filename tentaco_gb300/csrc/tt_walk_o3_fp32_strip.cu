// MTTKRP strip walk kernels, order 3, storage fp32.
#define TT_ORDER 3
#define TT_PREC kFP32
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o3_fp32_strip
#include "tt_walk_inst.cuh"
