// MTTKRP strip walk kernels, order 5, storage fx16.
#define TT_ORDER 5
#define TT_PREC kFX16
#define TT_STRIP_UNIT
#define TT_LOOKUP walk_launcher_o5_fx16_strip
#include "tt_walk_inst.cuh"
