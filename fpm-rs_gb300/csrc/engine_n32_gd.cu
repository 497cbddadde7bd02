// Gradient-descent and adaptive-AP engine instantiations for 32 x 32 tiles
// (the other families are in engine_n32.cu; the two build in parallel).
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(32, )
}  // namespace fpm
