// MTTKRP strip walk kernels, order 3, storage fx16.
#define TT_ORDER 3
#define TT_PREC kFX16
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o3_fx16_strip
#include "tt_walk_inst.cuh"
