// Gradient-descent and adaptive-AP engine instantiations for 256 x 256 tiles
// (the other families are in engine_n256.cu; the two build in parallel).
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(256, )
}  // namespace fpm
