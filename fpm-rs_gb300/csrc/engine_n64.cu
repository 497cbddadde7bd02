// Frame engine instantiation for 64 x 64 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(64, extern)  // in engine_n64_gd.cu
template struct EngineEntry<64>;
}  // namespace fpm
