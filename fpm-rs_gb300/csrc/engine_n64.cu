// Frame engine instantiation for 64 x 64 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
template struct EngineEntry<64>;
}  // namespace fpm
