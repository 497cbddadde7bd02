// Frame engine instantiation for 32 x 32 detector tiles.
#include "engine_impl.cuh"

namespace fpm {
template struct EngineEntry<32>;
}  // namespace fpm
