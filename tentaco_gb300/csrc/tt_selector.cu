// tt_selector.cu -- learned variant selector (placeholder until a model is loaded).
#include "tt_plan.h"
namespace tt {
int selector_pick(const tt_plan* p, const taco_tensor_t* B) {
  (void)p; (void)B;
  return -1;
}
}  // namespace tt
