// Size dispatch of the frame engine and its per-size helper kernels. The
// kernels themselves are in engine_impl.cuh, instantiated per tile size in
// engine_n32.cu, engine_n64.cu, engine_n128.cu and engine_n256.cu.
#include "engine_impl.cuh"

namespace fpm {

extern template struct EngineEntry<32>;
extern template struct EngineEntry<64>;
extern template struct EngineEntry<128>;
extern template struct EngineEntry<256>;

bool engine_supported(int n) { return n == 32 || n == 64 || n == 128 || n == 256; }

int engine_ctas(int n) {
    switch (n) {
        case 32: return Cfg<32>::C;
        case 64: return Cfg<64>::C;
        case 128: return Cfg<128>::C;
        case 256: return Cfg<256>::C;
        default: return 0;
    }
}

int engine_rows(int n) {
    switch (n) {
        case 32: return Cfg<32>::R;
        case 64: return Cfg<64>::R;
        case 128: return Cfg<128>::R;
        case 256: return Cfg<256>::R;
        default: return 0;
    }
}

int engine_na(int n) {
    switch (n) {
        case 32: return Cfg<32>::NA;
        case 64: return Cfg<64>::NA;
        case 128: return Cfg<128>::NA;
        case 256: return Cfg<256>::NA;
        default: return 0;
    }
}

int init_chunks(int n) { return (n * n + kInitBlock - 1) / kInitBlock; }

#define FPM_DISPATCH(call)                       \
    switch (n) {                                 \
        case 32: return EngineEntry<32>::call;   \
        case 64: return EngineEntry<64>::call;   \
        case 128: return EngineEntry<128>::call; \
        case 256: return EngineEntry<256>::call; \
        default: return cudaErrorInvalidValue;   \
    }

cudaError_t launch_engine(int n, const EngineParams& p, int tiles, cudaStream_t s) { FPM_DISPATCH(engine(p, tiles, s)) }

cudaError_t launch_forward(int n, const ForwardParams& p, cudaStream_t s) { FPM_DISPATCH(forward(p, s)) }

cudaError_t engine_max_active_clusters(int n, int* count) { FPM_DISPATCH(max_active_clusters(count)) }

cudaError_t launch_permute_f64_to_f32(int n, const double* src, float* dst, long long frames, cudaStream_t s) {
    FPM_DISPATCH(permute_f64(src, dst, frames, s))
}

cudaError_t launch_permute_u8(int n, const uint8_t* src, uint8_t* dst, long long frames, cudaStream_t s) {
    FPM_DISPATCH(permute_u8(src, dst, frames, s))
}

cudaError_t launch_unpermute_f32_to_f64(int n, const float* src, double* dst, long long frames, cudaStream_t s) {
    FPM_DISPATCH(unpermute_f64(src, dst, frames, s))
}

cudaError_t launch_init_mean(int n, int m, const InitTile* tiles, int count, double* avg, double* partial,
                             cudaStream_t s) {
    FPM_DISPATCH(init(m, tiles, count, avg, partial, s))
}

}  // namespace fpm
