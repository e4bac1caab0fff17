// MTTKRP strip walk kernels, order 5, storage fp16.
#define TT_ORDER 5
#define TT_PREC kFP16
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o5_fp16_strip
#include "tt_walk_inst.cuh"
