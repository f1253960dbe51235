// Mixed-model SQP launches of the built model pairs (a unit of its own so
// that it compiles in parallel with the single-model units).
#include "sqp_mixed.cuh"

namespace mpxg {

const MixedOps* mixed_ops(int model_a, int model_b) {
  if (model_a == MPXG_MODEL_SRBD_RPY12 && model_b == MPXG_MODEL_BIPED_WRENCH12)
    return &MixedLaunch<ModelRpy12, ModelBiped12>::ops();
  if (model_a == MPXG_MODEL_SRBD_QUAT13 && model_b == MPXG_MODEL_BIPED_WRENCH12)
    return &MixedLaunch<ModelQuat13, ModelBiped12>::ops();
  return nullptr;
}

}  // namespace mpxg
