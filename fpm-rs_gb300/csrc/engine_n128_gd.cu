// Gradient-descent and adaptive-AP engine instantiations for 128 x 128 tiles
// (the other families are in engine_n128.cu; the two build in parallel).
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(128, )
}  // namespace fpm
