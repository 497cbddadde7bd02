// fpm_fft2_noalloc: the Backend::fft2 transform of fpm_fft2 without any
// device allocation.
//
// Some callers cannot call cudaMalloc: a host whose device memory is owned by
// another allocator (a framework's caching pool or a serving loop that admits
// work by a fixed HBM budget, where an allocation the accounting does not see
// breaks the budget), and latency-sensitive loops for which cudaMalloc and
// cudaFree are off limits because they can synchronise the whole device. This
// entry point serves them with scratch that lives in one file-scope device
// array of fixed size, so nothing is allocated per call.
//
// The array holds kNoAllocMaxValues complex128 values (9 MiB) plus twiddle and
// factor tables; every GPU that loads this library keeps it until the process
// exits. Under CUDA's default lazy module loading the array is committed on
// the device by the first call there (its cudaGetSymbolAddress), with eager
// loading when the module loads: callers that budget device memory should make
// one call during their set-up so that those 9 MiB are taken before the budget
// is. All calls in the process share the array and it keeps the last call's
// contents; each call overwrites every element it reads, so nothing needs
// clearing. Calls that overlapped on the GPU would race on the array, so this
// entry point takes a process-wide lock (then the context's own lock, the
// order every caller keeps) and leaves nothing queued on the array when it
// returns, on success or error. The first call on each device looks up the
// array's device address with cudaGetSymbolAddress while that device is
// current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "fpm_gpu.h"
#include "kernels.h"

namespace {

constexpr long long kNoAllocMaxValues = 768LL * 768LL;  // complex128 values per transform
constexpr int kNoAllocMaxLine = 4096;                   // longest row or column
constexpr int kMaxFactors = 32;
constexpr int kMaxDevices = 64;

// Layout in double2 units: data | width roots | height roots | factor tables | pointer slot.
constexpr long long kRootsW = kNoAllocMaxValues;
constexpr long long kRootsH = kRootsW + kNoAllocMaxLine;
constexpr long long kFactors = kRootsH + kNoAllocMaxLine;  // 2 * kMaxFactors ints = kMaxFactors double2
constexpr long long kSlot = kFactors + kMaxFactors;
constexpr long long kScratchValues = kSlot + 1;

static __device__ __align__(256) double2 g_noalloc_scratch[kScratchValues];

std::mutex g_noalloc_lock;
double2* g_noalloc_address[kMaxDevices] = {};
double g_host_roots[2][2 * kNoAllocMaxLine];
int g_host_factors[2][kMaxFactors];

int factorise(int n, int* out) {
    int count = 0;
    for (int p = 2; (long long)p * p <= n; ++p)
        while (n % p == 0) {
            out[count++] = p;
            n /= p;
        }
    if (n > 1) out[count++] = n;
    return count;
}

void fill_roots(int n, double* out) {
    for (int k = 0; k < n; ++k) {
        const double a = 2.0 * M_PI * (double)k / (double)n;
        out[2 * k] = std::cos(a);
        out[2 * k + 1] = -std::sin(a);
    }
}

}  // namespace

extern "C" int32_t fpm_fft2_noalloc(fpm_context* ctx, double* values, int32_t height, int32_t width, int32_t inverse) {
    std::lock_guard<std::mutex> lock(g_noalloc_lock);
    char text[512];
    if (!ctx) {
        fpm::set_context_error(nullptr, "fpm_fft2_noalloc: context must be non-null");
        return FPM_ERR_INVALID_PARAMETER;
    }
    // The context's streams and error text belong to whichever entry point
    // holds its lock; this one takes it after the array's lock.
    std::lock_guard<std::mutex> context_lock(fpm::context_mutex(ctx));
    auto error = [&](int32_t code) {
        fpm::set_context_error(ctx, text);
        return code;
    };
    if (!values) {
        std::snprintf(text, sizeof text, "fpm_fft2_noalloc: values must be non-null");
        return error(FPM_ERR_INVALID_PARAMETER);
    }
    if (height <= 0 || width <= 0) {
        std::snprintf(text, sizeof text, "fpm_fft2_noalloc: FFT dimensions must be non-zero, got (%d, %d)", height,
                      width);
        return error(FPM_ERR_INVALID_SHAPE);
    }
    if ((long long)height * width > kNoAllocMaxValues || height > kNoAllocMaxLine || width > kNoAllocMaxLine) {
        std::snprintf(text, sizeof text,
                      "fpm_fft2_noalloc: shape (%d, %d) exceeds its fixed scratch: at most %lld values and %d per "
                      "row or column (use fpm_fft2 for larger transforms)",
                      height, width, kNoAllocMaxValues, kNoAllocMaxLine);
        return error(FPM_ERR_INVALID_SHAPE);
    }
    int device = 0;
    cudaStream_t s = nullptr;
    fpm::context_device_stream(ctx, &device, &s);
    // Once a copy or kernel is queued, an error return first waits for the
    // stream, so no work on the shared array outlives the lock.
    bool queued = false;
    auto cuda = [&](cudaError_t e, const char* what) {
        std::snprintf(text, sizeof text, "fpm_fft2_noalloc: %s failed: %s (%s)", what, cudaGetErrorName(e),
                      cudaGetErrorString(e));
        if (queued) (void)cudaStreamSynchronize(s);
        return error(FPM_ERR_CUDA);
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda(e, "cudaSetDevice");
    if (device < 0 || device >= kMaxDevices) {
        std::snprintf(text, sizeof text, "fpm_fft2_noalloc: device %d is beyond the supported %d devices", device,
                      kMaxDevices);
        return error(FPM_ERR_UNSUPPORTED);
    }
    if (!g_noalloc_address[device]) {
        // One-time set-up on this device: the array's device address.
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda(e, "cudaGetSymbolAddress");
        g_noalloc_address[device] = static_cast<double2*>(ptr);
    }
    double2* scratch = g_noalloc_address[device];
    double2* data = scratch;
    double2* roots_w = scratch + kRootsW;
    double2* roots_h = scratch + kRootsH;
    int* factors_w = reinterpret_cast<int*>(scratch + kFactors);
    int* factors_h = factors_w + kMaxFactors;
    double2** slot = reinterpret_cast<double2**>(scratch + kSlot);

    fill_roots(width, g_host_roots[0]);
    fill_roots(height, g_host_roots[1]);
    const int nfw = factorise(width, g_host_factors[0]);
    const int nfh = factorise(height, g_host_factors[1]);
    const size_t bytes = sizeof(double2) * (size_t)height * width;
    double2* host_slot = data;
    struct Copy {
        void* dst;
        const void* src;
        size_t bytes;
    } copies[] = {
        {data, values, bytes},
        {roots_w, g_host_roots[0], sizeof(double2) * (size_t)width},
        {roots_h, g_host_roots[1], sizeof(double2) * (size_t)height},
        {factors_w, g_host_factors[0], sizeof(int) * (size_t)(nfw > 0 ? nfw : 1)},
        {factors_h, g_host_factors[1], sizeof(int) * (size_t)(nfh > 0 ? nfh : 1)},
        {slot, &host_slot, sizeof(double2*)},
    };
    for (const Copy& c : copies) {
        e = cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyHostToDevice, s);
        queued = true;
        if (e != cudaSuccess) return cuda(e, "cudaMemcpyAsync (host to device)");
    }
    // Rows, then columns; the forward transform is scaled by 1/(h*w), as
    // CpuBackend::fft2 (src/backend/cpu.rs:130-175) does.
    e = fpm::launch_fft_lines(slot, 1, width, 1, width, height, inverse ? 1 : 0, roots_w, factors_w, nfw, 1.0, s);
    if (e != cudaSuccess) return cuda(e, "row transform launch");
    const double scale = inverse ? 1.0 : 1.0 / ((double)height * (double)width);
    e = fpm::launch_fft_lines(slot, 1, height, width, 1, width, inverse ? 1 : 0, roots_h, factors_h, nfh, scale, s);
    if (e != cudaSuccess) return cuda(e, "column transform launch");
    e = cudaMemcpyAsync(values, data, bytes, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda(e, "cudaMemcpyAsync (device to host)");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda(e, "cudaStreamSynchronize");
    return FPM_OK;
}
