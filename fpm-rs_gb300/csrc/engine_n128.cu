// Frame engine instantiation for 128 x 128 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
template struct EngineEntry<128>;
}  // namespace fpm
