// Frame engine instantiation for 128 x 128 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(128, extern)  // in engine_n128_gd.cu
template struct EngineEntry<128>;
}  // namespace fpm
