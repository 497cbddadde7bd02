// Gradient-descent and adaptive-AP engine instantiations for 64 x 64 tiles
// (the other families are in engine_n64.cu; the two build in parallel).
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(64, )
}  // namespace fpm
