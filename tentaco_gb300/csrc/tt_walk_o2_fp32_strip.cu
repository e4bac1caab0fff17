// Strip walk kernels over two levels (TTM: a tensor's fibers times one matrix), storage fp32.
#define TT_ORDER 2
#define TT_PREC kFP32
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o2_fp32_strip
#include "tt_walk_inst.cuh"
