// Frame engine instantiation for 256 x 256 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
template struct EngineEntry<256>;
}  // namespace fpm
