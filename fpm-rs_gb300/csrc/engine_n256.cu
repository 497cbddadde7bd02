// Frame engine instantiation for 256 x 256 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
FPM_ENGINE_SECOND_HALF(256, extern)  // in engine_n256_gd.cu
template struct EngineEntry<256>;
}  // namespace fpm
