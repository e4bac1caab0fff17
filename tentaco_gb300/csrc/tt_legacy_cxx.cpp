// tt_legacy_cxx.cpp -- the same reference entry points with C++ linkage.
//
// The reference declares them in gpu_kernels.cuh without extern "C", so objects
// compiled against that header reference the mangled names (for example
// _Z15mttkrp_gpu_tacoP13taco_tensor_tS0_S0_S0_).  This translation unit does
// not see the C-linkage declarations; it defines the C++ functions and
// forwards to the C-linkage implementation.
#include "../../include/tentaco/taco_tensor_t.h"

enum { TT_LEG_TACO = 0, TT_LEG_SR = 1, TT_LEG_PR = 2 };

extern "C" void tt_legacy_mttkrp(const char* name, int kind, int rank_in_name, int tb, int p1, int p2,
                                 taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
extern "C" void tt_legacy_ttv(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c);
extern "C" float tt_legacy_timer_ms(void);

__attribute__((visibility("default"))) float get_gpu_timer_result() { return tt_legacy_timer_ms(); }
__attribute__((visibility("default"))) void ttv_csf_gpu_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C) {
  tt_legacy_ttv(A, B, C);
}
#define X(name, kind, rank, tb, p1, p2)                                                      \
  __attribute__((visibility("default"))) void name(taco_tensor_t* A, taco_tensor_t* B,     \
                                                   taco_tensor_t* C, taco_tensor_t* D) {   \
    tt_legacy_mttkrp(#name, kind, rank, tb, p1, p2, A, B, C, D);                           \
  }
#include "../../include/tentaco/tt_legacy_names.def"
#undef X
