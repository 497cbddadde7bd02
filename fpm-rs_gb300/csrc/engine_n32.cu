// Frame engine instantiation for 32 x 32 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(32, extern)  // in engine_n32_gd.cu
template struct EngineEntry<32>;
}  // namespace fpm
