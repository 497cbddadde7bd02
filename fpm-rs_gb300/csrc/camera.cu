// Detector model on the device: CameraModel::measure_frame
// (src/simulation/camera.rs:249-290) applied to a whole forward stack.
//
// Random numbers come from a counter-based Philox-4x32-10 generator (Salmon,
// Moraes, Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC 2011): pixel e of a stack draws from its own counter stream (e, draw),
// keyed by the seed, so the counts do not depend on the launch shape.
// Poisson variates use inversion by sequential search below a mean of 10 and
// Hoermann's transformed rejection with squeeze (PTRS, "The transformed
// rejection method for generating Poisson random variables", Insurance:
// Mathematics and Economics 12, 1993) above; normal variates use the
// Box-Muller transform. The reference draws from ChaCha12 (rand 0.9), so
// counts agree with it in distribution, not value by value.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "kernels.h"

namespace fpm {
namespace {

__device__ __forceinline__ uint4 philox_round(uint4 c, uint2 k) {
    const unsigned m0 = 0xD2511F53u, m1 = 0xCD9E8D57u;
    const unsigned lo0 = m0 * c.x, hi0 = __umulhi(m0, c.x);
    const unsigned lo1 = m1 * c.z, hi1 = __umulhi(m1, c.z);
    return make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        c = philox_round(c, k);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Stream of uniforms for one pixel: block b of four 32-bit words is
// philox(counter = (pixel lo, pixel hi, b, 0), key = seed).
struct PixelStream {
    uint2 key;
    unsigned pixel_lo, pixel_hi;
    unsigned block = 0;
    uint4 words;
    int used = 4;

    __device__ unsigned next_word() {
        if (used == 4) {
            words = philox4x32_10(make_uint4(pixel_lo, pixel_hi, block++, 0u), key);
            used = 0;
        }
        const int i = used++;
        return i == 0 ? words.x : i == 1 ? words.y : i == 2 ? words.z : words.w;
    }
    // Uniform double in (0, 1): 53 random bits, offset by half a step.
    __device__ double uniform() {
        const unsigned long long hi = next_word(), lo = next_word();
        const unsigned long long bits = ((hi << 32) | lo) >> 11;
        return ((double)bits + 0.5) * 0x1.0p-53;
    }
    __device__ double normal() {
        const double u1 = uniform(), u2 = uniform();
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
};

constexpr int kMaxDraws = 1 << 16;  // bound on rejection loops (never reached in practice)

__device__ double poisson(PixelStream& rng, double lambda, int* status) {
    if (lambda < 10.0) {
        // Inversion: the smallest k with P(X <= k) >= u.
        const double u = rng.uniform();
        double p = exp(-lambda), cdf = p;
        int k = 0;
        while (u > cdf && k < kMaxDraws) {
            ++k;
            p *= lambda / k;
            cdf += p;
        }
        return (double)k;
    }
    const double slam = sqrt(lambda), loglam = log(lambda);
    const double b = 0.931 + 2.53 * slam;
    const double a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
    const double vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int draw = 0; draw < kMaxDraws; ++draw) {
        const double u = rng.uniform() - 0.5;
        const double v = rng.uniform();
        const double us = 0.5 - fabs(u);
        const double k = floor((2.0 * a / us + b) * u + lambda + 0.43);
        if (us >= 0.07 && v <= vr) return k;
        if (k < 0.0 || (us < 0.013 && v > us)) continue;
        if (log(v) + log(inv_alpha) - log(a / (us * us) + b) <= -lambda + k * loglam - lgamma(k + 1.0)) return k;
    }
    atomicOr(status, 1);
    return floor(lambda + 0.5);
}

__global__ void camera_kernel(const float* __restrict__ intensity, double* __restrict__ counts, long long total,
                              long long frame_len, CameraParams cp, int* status) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        PixelStream rng;
        rng.key = make_uint2((unsigned)cp.seed, (unsigned)(cp.seed >> 32));
        rng.pixel_lo = (unsigned)e;
        rng.pixel_hi = (unsigned)(e >> 32);
        const double sensitivity = cp.sensitivity ? cp.sensitivity[e % frame_len] : 1.0;
        const double expected = fmax((double)intensity[e], 0.0) * sensitivity * cp.photons_per_pixel + cp.dark_current;
        double electrons = cp.shot_noise && expected > 0.0 ? poisson(rng, expected, status) : expected;
        if (cp.read_noise > 0.0) electrons += cp.read_noise * rng.normal();
        double c = electrons * cp.gain_counts_per_electron + cp.offset_counts;
        c = fmin(fmax(c, 0.0), cp.maximum_count);
        if (cp.quantize) c = round(c);  // half away from zero, as f64::round
        counts[e] = c;
    }
}

}  // namespace

cudaError_t launch_camera(const float* intensity, double* counts, long long total, long long frame_len,
                          const CameraParams& params, int* status, cudaStream_t s) {
    if (total == 0) return cudaSuccess;
    const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    camera_kernel<<<blocks, 256, 0, s>>>(intensity, counts, total, frame_len, params, status);
    return cudaGetLastError();
}

}  // namespace fpm
