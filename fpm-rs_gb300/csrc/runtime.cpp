// Host runtime behind include/fpm_gpu.h: contexts, device-resident problems,
// model compilation, and the reconstruction runner. Control flow follows
// Runner::run (src/reconstruction/runner.rs:76-285): initialise the state,
// canonicalise (EPRY), iterate the schedule, canonicalise per iteration,
// record the weighted mean objective, and build the result. Every numerical
// step runs on the GPU; there is no host fallback.
#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's driver entry point)
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <chrono>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <vector>

#include <unistd.h>

#include "fpm_gpu.h"
#include "kernels.h"

namespace {

thread_local std::string g_global_error;

struct Status {
    int32_t code = FPM_OK;
    std::string message;
    static Status ok() { return Status(); }
    static Status make(int32_t c, const char* fmt, ...) {
        Status s;
        s.code = c;
        char buf[1024];
        va_list args;
        va_start(args, fmt);
        vsnprintf(buf, sizeof buf, fmt, args);
        va_end(args);
        s.message = buf;
        return s;
    }
    explicit operator bool() const { return code != FPM_OK; }
};

#define FPM_CUDA(call)                                                                                        \
    do {                                                                                                      \
        cudaError_t err_ = (call);                                                                            \
        if (err_ != cudaSuccess)                                                                              \
            return Status::make(FPM_ERR_CUDA, "CUDA error %s (%s) at %s:%d", cudaGetErrorName(err_),          \
                                cudaGetErrorString(err_), __FILE__, __LINE__);                                \
    } while (0)

#define FPM_TRY(expr)            \
    do {                         \
        Status st_ = (expr);     \
        if (st_) return st_;     \
    } while (0)

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    // Pooled buffers are stream-ordered allocations from the context's pool
    // on `stream`; others use cudaMalloc.
    cudaMemPool_t pool = nullptr;
    cudaStream_t stream = nullptr;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { release(); }
    // Later allocations and the free are ordered on s; an existing allocation
    // is kept (callers synchronise between runs on different streams).
    void bind(cudaMemPool_t p, cudaStream_t s) {
        if (ptr && p != pool) release();
        pool = p;
        stream = s;
    }
    void release() {
        if (ptr) {
            if (pool) cudaFreeAsync(ptr, stream);
            else cudaFree(ptr);
        }
        ptr = nullptr;
        bytes = 0;
    }
    Status ensure(size_t n) {
        if (n <= bytes && ptr) return Status::ok();
        release();
        if (n == 0) n = 16;
        if (pool) FPM_CUDA(cudaMallocFromPoolAsync(&ptr, n, pool, stream));
        else FPM_CUDA(cudaMalloc(&ptr, n));
        bytes = n;
        return Status::ok();
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(ptr);
    }
};

// Persistent host worker pool for the per-frame scans of problem creation:
// fn(i) for i in [0, count) on all hardware threads, the caller included.
// A forked child (the workers do not survive fork) runs serially.
class HostPool {
public:
    static HostPool& get() {
        static HostPool* pool = new HostPool();  // never destroyed: workers may still block at exit
        return *pool;
    }
    void run(long long count, const std::function<void(long long)>& fn) {
        if (count <= 0) return;
        if (workers_.empty() || count == 1 || getpid() != pid_) {
            for (long long i = 0; i < count; ++i) fn(i);
            return;
        }
        std::lock_guard<std::mutex> serial(run_mu_);
        {
            std::lock_guard<std::mutex> lk(mu_);
            task_ = &fn;
            count_ = count;
            next_.store(0);
            active_ = (int)workers_.size();
            ++generation_;
        }
        cv_.notify_all();
        drain(fn, count);
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return active_ == 0; });
        task_ = nullptr;
    }

private:
    HostPool() : pid_(getpid()) {
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        for (int w = 0; w + 1 < hw; ++w) workers_.emplace_back([this] { loop(); });
        for (auto& t : workers_) t.detach();
    }
    void drain(const std::function<void(long long)>& fn, long long count) {
        for (long long i; (i = next_.fetch_add(1)) < count;) fn(i);
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return generation_ != seen; });
            seen = generation_;
            const std::function<void(long long)>* fn = task_;
            const long long count = count_;
            lk.unlock();
            drain(*fn, count);
            lk.lock();
            if (--active_ == 0) done_.notify_all();
        }
    }
    pid_t pid_;
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_;
    const std::function<void(long long)>* task_ = nullptr;
    long long count_ = 0;
    std::atomic<long long> next_{0};
    int active_ = 0;
    unsigned long long generation_ = 0;
};

struct FftPlan {
    DeviceBuffer roots;
    DeviceBuffer factors;
    int nfactors = 0;
};

}  // namespace

// Pinned staging for host->device copies of caller (pageable) memory: host
// threads fill one slot while the copy engine drains the others. Pageable
// copies go through the driver's own staging on the calling thread alone.
struct PinnedRing {
    static constexpr int kSlots = 4;
    static constexpr size_t kSlotBytes = size_t(64) << 20;
    void* slot[kSlots] = {};
    // Per slot, the last copy from it on each stream that used it.
    std::vector<std::pair<cudaStream_t, cudaEvent_t>> pending[kSlots];
    std::vector<cudaEvent_t> spare;
    int cur = 0;      // slot being filled
    size_t used = 0;  // bytes of it handed out (256-byte granules)
    ~PinnedRing() {
        for (int k = 0; k < kSlots; ++k) {
            for (auto& pe : pending[k]) {
                cudaEventSynchronize(pe.second);
                cudaEventDestroy(pe.second);
            }
            if (slot[k]) cudaFreeHost(slot[k]);
        }
        for (cudaEvent_t e : spare) cudaEventDestroy(e);
    }
};

struct fpm_context {
    int device = 0;
    static constexpr int kStreams = 4;
    cudaStream_t streams[kStreams] = {};
    std::string error;
    std::mutex mu;
    std::map<int, std::unique_ptr<FftPlan>> plans;
    DeviceBuffer scratch_a, scratch_b;
    cudaMemPool_t pool = nullptr;  // problem buffers: stream-ordered, memory kept for reuse
    cudaStream_t upload = nullptr, download = nullptr;  // host-input batches: copies beside compute
    fpm_run_stats stats = {};
    // Clusters of a frame-engine launch per tile size (index log2(n) - 5; 0:
    // one cluster per tile); with fewer, each cluster walks several tiles.
    int engine_grid[4] = {0, 0, 0, 0};
    // Frame-engine shape per tile size (FPM_ENGINE_CLUSTER, _SINGLE_CTA or
    // _AUTO).
    int engine_shape[4] = {FPM_ENGINE_CLUSTER, FPM_ENGINE_CLUSTER, FPM_ENGINE_CLUSTER, FPM_ENGINE_AUTO};
    // CTAs of a single-CTA engine launch per tile size (0: as many as fit at once).
    int engine_ctas[4] = {0, 0, 0, 0};
    std::unique_ptr<PinnedRing> pinned;  // created by the first large upload
};

struct fpm_problem {
    fpm_context* ctx = nullptr;
    int n = 0, m = 0, frames = 0;
    std::vector<int64_t> start_row, start_col;
    std::vector<double> off_row, off_col, kx, ky, gains, weights, data_snr;
    std::vector<uint8_t> support;
    std::vector<double> pupil;  // complex128 interleaved
    std::vector<double> upload_gains;  // host sources of asynchronous uploads
    std::vector<float2> pupil_f32;
    std::vector<int2> pupil_spans;  // host source of pupil_span
    bool unit_pupil = false;  // pupil_f32 is exactly 1 on one column interval per row and 0 elsewhere
    int host_status = 0;                // result downloads
    std::vector<double> host_partials;
    int it0 = 0;                        // first iteration of the last run (resumed runs start later)
    std::vector<double> resume_objectives;
    int host_counter = 0;
    std::vector<fpm::FrameParam> params;
    std::vector<double> stencil_cells;  // per frame: rows * cols of the bilinear stencil
    bool has_masks = false, has_background = false;
    bool amplitude = false;  // device measurements hold sqrt(max(I / g, 0)), -1 where masked
    long long background_stride = 0;
    bool row_exact = true, col_exact = true;
    double weight_sum = 0.0;
    // resident device data
    DeviceBuffer meas, masks, background, frame_params, support_d, pupil_ref, pupil_model, pupil_span, gains_d;
    std::vector<double> state_gains;  // host source of gains_d: the model gains (1 where not positive)
    // run state
    DeviceBuffer object, pupil_state, velocity, anchor, partials, counter, status, scratch64, order, gradient,
        object_err, gradient_err,
        pupil_gradient, tv_scratch, pupil_scratch;
    // GD illumination recovery: the run's frame constants, crop starts and
    // offsets, corrections and per-CTA gradient partials.
    DeviceBuffer ill_params, ill_start, ill_offset, ill_correction, ill_partials;
    // EPRY frame-gain and background recovery: state gains [frames], state
    // backgrounds [frames][N * N] (engine layout), and their natural-order
    // FP64 copy for downloads.
    DeviceBuffer gain_state, bg_state, bg_natural;
    fpm_job* busy = nullptr;  // the submitted job that owns the problem until it finishes
    fpm_plan* plan = nullptr;  // the captured run plan that holds the problem until destroyed
};

namespace {

// The context's pinned ring, created on first use.
Status pinned_ring(fpm_context* ctx, PinnedRing** out) {
    if (!ctx->pinned) {
        auto ring = std::make_unique<PinnedRing>();
        for (int k = 0; k < PinnedRing::kSlots; ++k)
            FPM_CUDA(cudaHostAlloc(&ring->slot[k], PinnedRing::kSlotBytes, cudaHostAllocDefault));
        ctx->pinned = std::move(ring);
    }
    *out = ctx->pinned.get();
    return Status::ok();
}

// `len` bytes (at most a slot) of the ring's current slot, moving to the
// next slot, once the copies from it on every stream have finished, when
// the current one is full.
Status ring_take(PinnedRing& R, size_t len, char** at) {
    if (R.used + len > PinnedRing::kSlotBytes) {
        R.cur = (R.cur + 1) % PinnedRing::kSlots;
        R.used = 0;
        for (auto& pe : R.pending[R.cur]) {
            FPM_CUDA(cudaEventSynchronize(pe.second));
            R.spare.push_back(pe.second);
        }
        R.pending[R.cur].clear();
    }
    *at = static_cast<char*>(R.slot[R.cur]) + R.used;
    R.used += (len + 255) & ~size_t(255);
    return Status::ok();
}

// Queues the copy of `len` bytes at `at` (in the current slot) to `dst` on
// stream s and records it against the slot.
Status ring_copy(PinnedRing& R, void* dst, const char* at, size_t len, cudaStream_t s) {
    FPM_CUDA(cudaMemcpyAsync(dst, at, len, cudaMemcpyHostToDevice, s));
    auto& pend = R.pending[R.cur];
    auto it = std::find_if(pend.begin(), pend.end(), [&](const auto& pe) { return pe.first == s; });
    if (it == pend.end()) {
        cudaEvent_t e = nullptr;
        if (!R.spare.empty()) {
            e = R.spare.back();
            R.spare.pop_back();
        } else {
            FPM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        pend.emplace_back(s, e);
        it = pend.end() - 1;
    }
    FPM_CUDA(cudaEventRecord(it->second, s));  // a stream's copies complete in order
    return Status::ok();
}

// Host -> device copy of `bytes` of pageable memory on stream s, through
// the context's pinned ring. A copy straight from pageable memory first
// waits for all earlier work on its stream, so the host would stall behind
// the device at every small table; here each copy takes the next free
// stretch of the current slot, large ones in 64 MB pieces copied by the host
// worker pool. The caller holds the context.
Status upload_pageable(fpm_context* ctx, void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return Status::ok();
    PinnedRing* ring = nullptr;
    FPM_TRY(pinned_ring(ctx, &ring));
    constexpr size_t kPiece = size_t(1) << 20;
    for (size_t off = 0; off < bytes;) {
        const size_t len = std::min(bytes - off, PinnedRing::kSlotBytes);
        char* at = nullptr;
        FPM_TRY(ring_take(*ring, len, &at));
        const char* from = static_cast<const char*>(src) + off;
        if (len <= kPiece) {
            std::memcpy(at, from, len);
        } else {
            HostPool::get().run((long long)((len + kPiece - 1) / kPiece), [&](long long q) {
                const size_t o = (size_t)q * kPiece;
                std::memcpy(at + o, from + o, std::min(kPiece, len - o));
            });
        }
        FPM_TRY(ring_copy(*ring, static_cast<char*>(dst) + off, at, len, s));
        off += len;
    }
    return Status::ok();
}

// Host -> device copy of `rows` rows of `row_bytes` each, produced on the
// host straight into the pinned ring: fill(row, out) writes row `row` at
// `out`, in parallel over the host worker pool. Nothing runs on the device
// but the copies, so an upload never waits for an SM behind the persistent
// engine launches. The caller holds the context.
Status upload_rows(fpm_context* ctx, void* dst, long long rows, size_t row_bytes, cudaStream_t s,
                   const std::function<void(long long, char*)>& fill) {
    if (rows <= 0) return Status::ok();
    PinnedRing* ring = nullptr;
    FPM_TRY(pinned_ring(ctx, &ring));
    const long long per_slot = std::max<long long>(1, (long long)(PinnedRing::kSlotBytes / row_bytes));
    constexpr long long kRowsPerTask = 16;
    for (long long r0 = 0; r0 < rows;) {
        const long long n = std::min(per_slot, rows - r0);
        const size_t len = (size_t)n * row_bytes;
        char* at = nullptr;
        FPM_TRY(ring_take(*ring, len, &at));
        HostPool::get().run((n + kRowsPerTask - 1) / kRowsPerTask, [&](long long q) {
            const long long a = q * kRowsPerTask, b = std::min(n, a + kRowsPerTask);
            for (long long r = a; r < b; ++r) fill(r0 + r, at + (size_t)r * row_bytes);
        });
        FPM_TRY(ring_copy(*ring, static_cast<char*>(dst) + (size_t)r0 * row_bytes, at, len, s));
        r0 += n;
    }
    return Status::ok();
}

Status set_error(fpm_context* ctx, Status s) {
    if (ctx) ctx->error = s.message;
    g_global_error = s.message;
    return s;
}

int32_t finish(fpm_context* ctx, const Status& s) {
    if (s) set_error(ctx, s);
    return s.code;
}

// ------------------------------------------------------------ geometry

struct GridShift {
    long long integer;
    double offset;
    long long lower, upper;
};

// checked_grid_shift (src/model/image_plane_fpm.rs:975-1024).
Status grid_shift(double value, GridShift& g) {
    if (!std::isfinite(value)) return Status::make(FPM_ERR_INVALID_MODEL, "illumination shift must be finite");
    const double rounded = std::round(value);
    g.integer = (long long)rounded;
    g.offset = value - rounded;
    const double nearest = std::round(g.offset);
    if (std::fabs(g.offset - nearest) <= 1e-12) {
        g.lower = g.upper = g.integer + (long long)nearest;
    } else if (g.offset > 0.0) {
        g.lower = g.integer;
        g.upper = g.integer + 1;
    } else {
        g.lower = g.integer - 1;
        g.upper = g.integer;
    }
    return Status::ok();
}

struct Axis {
    long long lower_start;
    bool upper;
    double lower_weight, upper_weight;
};

// interpolation_axis (src/model/crop.rs:266-313).
Status interpolation_axis(long long start, long long length, long long bound, double offset, Axis& a) {
    if (length == 0 || bound == 0 || !std::isfinite(offset))
        return Status::make(FPM_ERR_INVALID_MODEL, "subpixel crop dimensions and offset must be finite and non-zero");
    const double nearest = std::round(offset);
    double integer_offset, fraction;
    if (std::fabs(offset - nearest) <= 1e-12) {
        integer_offset = nearest;
        fraction = 0.0;
    } else {
        integer_offset = std::floor(offset);
        fraction = offset - integer_offset;
    }
    const long long lower = start + (long long)integer_offset;
    if (lower < 0) return Status::make(FPM_ERR_INVALID_MODEL, "subpixel crop starts outside the grid");
    const long long end = lower + length;
    const bool upper = fraction > 0.0;
    if (end > bound || (upper && end >= bound))
        return Status::make(FPM_ERR_INVALID_MODEL, "subpixel crop interpolation stencil lies outside the grid");
    a.lower_start = lower;
    a.upper = upper;
    a.lower_weight = 1.0 - fraction;
    a.upper_weight = fraction;
    return Status::ok();
}

Status validate_optics(const fpm_optics& o) {
    const double v[6] = {o.wavelength_vacuum_m, o.objective_na, o.magnification, o.camera_pixel_size,
                         o.illumination_refractive_index, o.objective_medium_refractive_index};
    const char* names[6] = {"wavelength_vacuum_m", "objective_na", "magnification", "camera_pixel_size",
                            "illumination_refractive_index", "objective_medium_refractive_index"};
    for (int i = 0; i < 6; ++i)
        if (!std::isfinite(v[i]) || v[i] <= 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "%s must be finite and positive, got %g", names[i], v[i]);
    if (o.objective_na > o.objective_medium_refractive_index)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "objective_na cannot exceed the medium refractive index");
    const double pixel = o.camera_pixel_size / o.magnification;
    const double limit = o.wavelength_vacuum_m / (2.0 * o.objective_na);
    if (!(pixel < limit))
        return Status::make(FPM_ERR_INVALID_PARAMETER,
                            "object-plane pitch camera_pixel_size / magnification (%.6e m) must be strictly less than "
                            "wavelength_vacuum_m / (2 * objective_na) (%.6e m)",
                            pixel, limit);
    if (o.has_defocus && !std::isfinite(o.defocus_distance))
        return Status::make(FPM_ERR_INVALID_PARAMETER, "defocus_distance must be finite");
    if (o.has_aberration) {
        if (!std::isfinite(o.astigmatism) || !std::isfinite(o.coma) || !std::isfinite(o.spherical) ||
            !std::isfinite(o.edge_apodization) || o.edge_apodization < 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "pupil_aberration coefficients are invalid");
    }
    return Status::ok();
}

struct Bounds {
    long long min_row, max_row, min_col, max_col;
};

Status displacement_bounds(const fpm_optics& o, int n, const double* kx, const double* ky, int h, int w, Bounds& b) {
    if (h <= 0 || w <= 0) return Status::make(FPM_ERR_INVALID_SHAPE, "image shape (%d, %d) must be non-zero", h, w);
    if (n <= 0) return Status::make(FPM_ERR_INVALID_MODEL, "illumination must contain at least one frame");
    const double pixel = o.camera_pixel_size / o.magnification;
    const double dkx = 2.0 * M_PI / ((double)w * pixel), dky = 2.0 * M_PI / ((double)h * pixel);
    b = {LLONG_MAX, LLONG_MIN, LLONG_MAX, LLONG_MIN};
    for (int i = 0; i < n; ++i) {
        GridShift r{}, c{};
        FPM_TRY(grid_shift(ky[i] / dky, r));
        FPM_TRY(grid_shift(kx[i] / dkx, c));
        b.min_row = std::min(b.min_row, r.lower);
        b.max_row = std::max(b.max_row, r.upper);
        b.min_col = std::min(b.min_col, c.lower);
        b.max_col = std::max(b.max_col, c.upper);
    }
    return Status::ok();
}

bool axis_contains(long long len, long long recon, long long lo, long long hi) {
    const long long base = recon / 2 - len / 2;
    return base + lo >= 0 && base + (len - 1) + hi < recon;
}

bool fits(int h, int w, long long mh, long long mw, const Bounds& b) {
    return axis_contains(h, mh, b.min_row, b.max_row) && axis_contains(w, mw, b.min_col, b.max_col);
}

void smooth_visit(long long value, int prime, long long minimum, long long& best) {
    static const long long primes[4] = {2, 3, 5, 7};
    if (value >= minimum) {
        if (best < 0 || value < best) best = value;
        return;
    }
    for (int i = prime; i < 4; ++i) {
        const long long next = value * primes[i];
        if (best < 0 || next < best) smooth_visit(next, i, minimum, best);
    }
}

// resolve_reconstruction_shape (src/model/image_plane_fpm.rs:287-348).
Status resolve_shape(int h, int w, int policy, int& mh, int& mw, const Bounds& b) {
    if (policy == FPM_SHAPE_EXACT) {
        if (mh < h || mw < w)
            return Status::make(FPM_ERR_INVALID_SHAPE, "image shape (%d, %d) must fit reconstruction shape (%d, %d)", h,
                                w, mh, mw);
        if ((long long)mh * w != (long long)mw * h)
            return Status::make(FPM_ERR_INVALID_SHAPE, "reconstruction must use the same scale factor in both dimensions");
        if (!fits(h, w, mh, mw, b))
            return Status::make(FPM_ERR_INVALID_SHAPE,
                                "reconstruction shape (%d, %d) does not contain every illumination crop and subpixel "
                                "interpolation stencil",
                                mh, mw);
        return Status::ok();
    }
    if (policy < 0 || policy > 3) return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown reconstruction shape policy");
    const long long d = std::gcd((long long)h, (long long)w);
    const long long ah = h / d, aw = w / d;
    const long long maximum = 1LL << 30;
    long long mult;
    if (fits(h, w, ah * d, aw * d, b)) {
        mult = d;
    } else {
        long long lower = d, upper = d;
        for (;;) {
            upper = std::min(upper * 2, maximum);
            if (upper == lower)
                return Status::make(FPM_ERR_INVALID_SHAPE,
                                    "illumination crops require a reconstruction shape outside the supported index range");
            if (fits(h, w, ah * upper, aw * upper, b)) break;
            lower = upper;
        }
        while (lower + 1 < upper) {
            const long long mid = lower + (upper - lower) / 2;
            if (fits(h, w, ah * mid, aw * mid, b))
                upper = mid;
            else
                lower = mid;
        }
        mult = upper;
    }
    if (policy == FPM_SHAPE_SMOOTH) {
        long long best = -1;
        smooth_visit(1, 0, mult, best);
        mult = best;
    } else if (policy == FPM_SHAPE_POWER_OF_TWO) {
        long long p = 1;
        while (p < mult) p <<= 1;
        mult = p;
    }
    mh = (int)(ah * mult);
    mw = (int)(aw * mult);
    return Status::ok();
}

// ------------------------------------------------------------- FFT plans

std::vector<int> prime_factors(int n) {
    std::vector<int> f;
    for (int p = 2; (long long)p * p <= n; ++p)
        while (n % p == 0) {
            f.push_back(p);
            n /= p;
        }
    if (n > 1) f.push_back(n);
    return f;
}

Status get_plan(fpm_context* ctx, int n, FftPlan*& out) {
    auto it = ctx->plans.find(n);
    if (it != ctx->plans.end()) {
        out = it->second.get();
        return Status::ok();
    }
    if (n > 4096) return Status::make(FPM_ERR_UNSUPPORTED, "FP64 line FFT supports lengths up to 4096, got %d", n);
    auto plan = std::make_unique<FftPlan>();
    std::vector<double> roots(2 * (size_t)n);
    for (int k = 0; k < n; ++k) {
        const double a = 2.0 * M_PI * (double)k / (double)n;
        roots[2 * k] = std::cos(a);
        roots[2 * k + 1] = -std::sin(a);
    }
    std::vector<int> f = prime_factors(n);
    FPM_TRY(plan->roots.ensure(roots.size() * sizeof(double)));
    FPM_TRY(plan->factors.ensure(std::max<size_t>(f.size(), 1) * sizeof(int)));
    // Stream-ordered copies: a synchronous copy would also wait for device work in flight.
    cudaStream_t s = ctx->streams[0];
    FPM_CUDA(cudaMemcpyAsync(plan->roots.ptr, roots.data(), roots.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    if (!f.empty())
        FPM_CUDA(cudaMemcpyAsync(plan->factors.ptr, f.data(), f.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    FPM_CUDA(cudaStreamSynchronize(s));
    plan->nfactors = (int)f.size();
    out = plan.get();
    ctx->plans[n] = std::move(plan);
    return Status::ok();
}

// Forward (scaled by 1/(h*w)) or inverse 2-D transform of `count` natural
// FP64 arrays of shape (h, w): rows, then columns, as CpuBackend::fft2.
Status fft2_device(fpm_context* ctx, double2* const* arrays_dev, int count, int h, int w, bool inverse,
                   cudaStream_t s) {
    FftPlan* pw = nullptr;
    FftPlan* ph = nullptr;
    FPM_TRY(get_plan(ctx, w, pw));
    FPM_TRY(get_plan(ctx, h, ph));
    FPM_CUDA(fpm::launch_fft_lines(arrays_dev, count, w, 1, w, h, inverse ? 1 : 0, pw->roots.as<double2>(),
                                   pw->factors.as<int>(), pw->nfactors, 1.0, s));
    const double scale = inverse ? 1.0 : 1.0 / ((double)h * (double)w);
    FPM_CUDA(fpm::launch_fft_lines(arrays_dev, count, h, w, 1, w, inverse ? 1 : 0, ph->roots.as<double2>(),
                                   ph->factors.as<int>(), ph->nfactors, scale, s));
    return Status::ok();
}

// ------------------------------------------------------------- problems

Status validate_model(const fpm_model_desc* md) {
    if (!md) return Status::make(FPM_ERR_INVALID_MODEL, "model descriptor is null");
    const int h = md->image_height, w = md->image_width;
    if (h <= 0 || w <= 0) return Status::make(FPM_ERR_INVALID_SHAPE, "image shape (%d, %d) must be non-zero", h, w);
    if (md->recon_height < h || md->recon_width < w)
        return Status::make(FPM_ERR_INVALID_MODEL, "reconstruction shape must contain a low-resolution crop");
    if (md->sources <= 0) return Status::make(FPM_ERR_INVALID_MODEL, "0 source k-vectors and crops; counts must be equal and non-zero");
    if (!md->crop_start_row || !md->crop_start_col || !md->pupil || !md->support)
        return Status::make(FPM_ERR_INVALID_MODEL, "model crops, pupil and support are required");
    const size_t n = (size_t)h * w;
    for (size_t i = 0; i < n; ++i) {
        if (!std::isfinite(md->pupil[2 * i]) || !std::isfinite(md->pupil[2 * i + 1]) || md->support[i] > 1)
            return Status::make(FPM_ERR_INVALID_MODEL, "pupil support or numeric values are invalid");
    }
    for (int s = 0; s < md->sources; ++s) {
        const long long sr = md->crop_start_row[s], sc = md->crop_start_col[s];
        if (sr < 0 || sc < 0 || sr + h > md->recon_height || sc + w > md->recon_width)
            return Status::make(FPM_ERR_INVALID_MODEL, "crop %d lies outside reconstruction shape", s);
        const double orow = md->offset_row ? md->offset_row[s] : 0.0;
        const double ocol = md->offset_col ? md->offset_col[s] : 0.0;
        Axis a{};
        FPM_TRY(interpolation_axis(sr, h, md->recon_height, orow, a));
        FPM_TRY(interpolation_axis(sc, w, md->recon_width, ocol, a));
        if (md->frame_gains && (!std::isfinite(md->frame_gains[s]) || md->frame_gains[s] < 0.0))
            return Status::make(FPM_ERR_INVALID_MODEL, "frame gains must be finite and non-negative");
    }
    if (md->background) {
        if (md->background_len != (int64_t)n && md->background_len != (int64_t)n * md->sources)
            return Status::make(FPM_ERR_INVALID_MODEL, "background must be one image or one image per frame");
        for (int64_t i = 0; i < md->background_len; ++i)
            if (!std::isfinite(md->background[i]))
                return Status::make(FPM_ERR_INVALID_MODEL, "background values must be finite");
    }
    return Status::ok();
}

// Header checks of a measurement stack that need no pass over the pixels.
Status check_measurement_header(const fpm_model_desc* md, const fpm_measurement_desc* ms) {
    if (!ms || !ms->measurements) return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "measurements are required");
    if (ms->frames != md->sources)
        return Status::make(FPM_ERR_INVALID_MODEL, "%d measurement frames but %d model frames", ms->frames, md->sources);
    int positive = 0;
    for (int f = 0; f < ms->frames; ++f) {
        const double wgt = ms->frame_weights ? ms->frame_weights[f] : 1.0;
        if (!std::isfinite(wgt) || wgt < 0.0)
            return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "frame %d has invalid weight %g", f, wgt);
        if (wgt > 0.0) ++positive;
    }
    if (positive == 0) return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "at least one frame must have positive weight");
    const int h = md->image_height, w = md->image_width;
    if (h != w || !fpm::engine_supported(h))
        return Status::make(FPM_ERR_UNSUPPORTED,
                            "the GB300 device path supports square detector frames of 32, 64, 128 or 256 pixels, got (%d, %d)",
                            h, w);
    if (md->recon_height != md->recon_width)
        return Status::make(FPM_ERR_UNSUPPORTED, "the GB300 device path supports square reconstruction grids");
    return Status::ok();
}

// One pass over a frame's pixels: finiteness, the unmasked count, and the
// snr_weighted score weight * sqrt(mean over unmasked pixels of
// max(I - background, 0)) (src/reconstruction/schedule.rs:104-128), summed in
// pixel order.
struct FrameScan {
    bool finite = true, any_unmasked = true;
    long long valid = 0;
    double snr = 0.0;
};

void scan_frame(const fpm_model_desc* md, const fpm_measurement_desc* ms, int f, FrameScan& out) {
    const size_t n2 = (size_t)md->image_height * md->image_width;
    const double* m = ms->measurements + (size_t)f * n2;
    const uint8_t* mk = ms->masks ? ms->masks + (size_t)f * n2 : nullptr;
    const double weight = ms->frame_weights ? ms->frame_weights[f] : 1.0;
    const long long bg_stride = (md->background && md->background_len != (int64_t)n2) ? (long long)n2 : 0;
    const double* bg = md->background ? md->background + (size_t)f * bg_stride : nullptr;
    bool finite = true;
    long long valid = 0;
    double sum = 0.0;
    for (size_t i = 0; i < n2; ++i) {
        const double v = m[i];
        finite &= std::isfinite(v);
        if (mk && mk[i] == 0) continue;
        ++valid;
        sum += std::max(v - (bg ? bg[i] : 0.0), 0.0);
    }
    out.finite = finite;
    out.valid = valid;
    out.any_unmasked = valid > 0;
    out.snr = weight == 0.0 || valid == 0 ? -INFINITY : weight * std::sqrt(sum / (double)valid);
}

Status check_scans(const fpm_measurement_desc* ms, const FrameScan* scans) {
    for (int f = 0; f < ms->frames; ++f)
        if (!scans[f].finite) return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "measurements contain non-finite values");
    for (int f = 0; f < ms->frames; ++f) {
        const double wgt = ms->frame_weights ? ms->frame_weights[f] : 1.0;
        if (wgt > 0.0 && ms->masks && !scans[f].any_unmasked)
            return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "positive-weight frame %d has no unmasked pixels", f);
    }
    return Status::ok();
}

// Bilinear stencil of one source's crop (interpolation_axis,
// src/model/crop.rs:266-313; extract_standard :79-102 for integer offsets),
// FP64 on the host, weights rounded once.
Status crop_frame_param(long long start_row, long long start_col, double off_row, double off_col, int N, int M,
                        fpm::FrameParam& fp) {
    Axis r{}, c{};
    FPM_TRY(interpolation_axis(start_row, N, M, off_row, r));
    FPM_TRY(interpolation_axis(start_col, N, M, off_col, c));
    fp = fpm::FrameParam{};
    if (std::fabs(off_row) <= 1e-12 && std::fabs(off_col) <= 1e-12) {
        fp.lower_row = (int)start_row;
        fp.lower_col = (int)start_col;
        fp.has_upper_row = fp.has_upper_col = 0;
        fp.w00 = 1.f;
        fp.w01 = fp.w10 = fp.w11 = 0.f;
    } else {
        fp.lower_row = (int)r.lower_start;
        fp.lower_col = (int)c.lower_start;
        fp.has_upper_row = r.upper ? 1 : 0;
        fp.has_upper_col = c.upper ? 1 : 0;
        fp.w00 = (float)(r.lower_weight * c.lower_weight);
        fp.w01 = (float)(r.lower_weight * c.upper_weight);
        fp.w10 = (float)(r.upper_weight * c.lower_weight);
        fp.w11 = (float)(r.upper_weight * c.upper_weight);
    }
    return Status::ok();
}

// Host part of a problem: copies of the model and the frame constants.
Status prepare_problem(fpm_context* ctx, const fpm_model_desc* md, const fpm_measurement_desc* ms,
                       const FrameScan* scans, std::unique_ptr<fpm_problem>& out) {
    auto p = std::make_unique<fpm_problem>();
    p->ctx = ctx;
    p->n = md->image_height;
    p->m = md->recon_height;
    p->frames = ms->frames;
    const int N = p->n, F = ms->frames;
    const size_t n2 = (size_t)N * N;
    const bool masks = ms->masks != nullptr;
    p->start_row.assign(md->crop_start_row, md->crop_start_row + F);
    p->start_col.assign(md->crop_start_col, md->crop_start_col + F);
    p->off_row.assign(F, 0.0);
    p->off_col.assign(F, 0.0);
    if (md->offset_row) p->off_row.assign(md->offset_row, md->offset_row + F);
    if (md->offset_col) p->off_col.assign(md->offset_col, md->offset_col + F);
    p->kx.assign(F, 0.0);
    p->ky.assign(F, 0.0);
    if (md->kx) p->kx.assign(md->kx, md->kx + F);
    if (md->ky) p->ky.assign(md->ky, md->ky + F);
    p->gains.assign(F, 1.0);
    if (md->frame_gains) p->gains.assign(md->frame_gains, md->frame_gains + F);
    p->weights.assign(F, 1.0);
    if (ms->frame_weights) p->weights.assign(ms->frame_weights, ms->frame_weights + F);
    p->support.assign(md->support, md->support + n2);
    p->pupil.assign(md->pupil, md->pupil + 2 * n2);
    p->has_masks = masks;
    p->has_background = md->background != nullptr;
    p->background_stride = (md->background && md->background_len != (int64_t)n2) ? (long long)n2 : 0;
    p->amplitude = md->background == nullptr;

    // Frame constants (FP64 on the host, rounded once).
    p->params.resize(F);
    p->stencil_cells.resize(F);
    p->data_snr.resize(F);
    for (int f = 0; f < F; ++f) p->data_snr[f] = scans[f].snr;
    for (int f = 0; f < F; ++f) {
        if (std::fabs(p->off_row[f]) > 1e-12) p->row_exact = false;
        if (std::fabs(p->off_col[f]) > 1e-12) p->col_exact = false;
        fpm::FrameParam fp{};
        FPM_TRY(crop_frame_param(p->start_row[f], p->start_col[f], p->off_row[f], p->off_col[f], N, p->m, fp));
        p->stencil_cells[f] = (double)(N + fp.has_upper_row) * (double)(N + fp.has_upper_col);
        const long long valid = masks ? scans[f].valid : (long long)n2;
        fp.weight = (float)p->weights[f];
        if (p->weights[f] > 0.0 && !(p->gains[f] > 0.0))
            return Status::make(FPM_ERR_INVALID_MODEL, "state frame %d has invalid gain %g", f, p->gains[f]);
        fp.gain = (float)(p->gains[f] > 0.0 ? p->gains[f] : 1.0);
        fp.valid_scale = valid > 0 ? (float)((double)n2 / (double)valid) : 0.f;
        fp.loss_scale = valid > 0 ? p->weights[f] / (double)valid : 0.0;
        p->params[f] = fp;
        p->weight_sum += p->weights[f];
    }

    out = std::move(p);
    return Status::ok();
}

// Device part: allocations from the context's pool and uploads on stream s.
// FP64 staging comes from the pool too and is freed stream-ordered once
// permuted, so uploads never wait for one another or for device work in
// flight; host vectors copied from live in the problem.
Status upload_problem(fpm_context* ctx, fpm_problem* p, const fpm_model_desc* md, const fpm_measurement_desc* ms,
                      cudaStream_t s) {
    const int N = p->n, F = p->frames;
    const size_t n2 = (size_t)N * N;
    for (DeviceBuffer* b : {&p->meas, &p->masks, &p->background, &p->frame_params, &p->support_d, &p->pupil_ref,
                            &p->pupil_model, &p->pupil_span, &p->gains_d})
        b->bind(ctx->pool, s);
    // Measurements go to the engine's FP32 layout, converted and permuted on
    // the host into the pinned ring (engine row e of a frame holds natural
    // row e / R + C (e % R); its position t holds natural column
    // t / NB + NA (t % NB)). With no background the engine reads the
    // amplitude form sqrt(max(I / g, 0)) (-1 on masked pixels): one float
    // per pixel, no mask bytes, and no divide or square root in the frame
    // loop. Every upload path converts the same way, so results do not
    // depend on how a problem was uploaded.
    const size_t total = n2 * F;
    const int C = fpm::engine_ctas(N), R = fpm::engine_rows(N), NA = fpm::engine_na(N), NB = N / NA;
    std::vector<int> column(N);
    for (int t = 0; t < N; ++t) column[t] = t / NB + NA * (t % NB);
    auto natural_row = [=](long long e) { return (int)(e / R) + C * (int)(e % R); };
    FPM_TRY(p->meas.ensure(total * sizeof(float)));
    if (p->amplitude) {
        p->upload_gains.resize(F);
        for (int f = 0; f < F; ++f) p->upload_gains[f] = p->gains[f] > 0.0 ? p->gains[f] : 1.0;
        const double* gains = p->upload_gains.data();
        FPM_TRY(upload_rows(ctx, p->meas.ptr, (long long)F * N, N * sizeof(float), s, [&](long long row, char* out) {
            const long long f = row / N;
            const size_t base = ((size_t)f * N + natural_row(row % N)) * N;
            const double* in = ms->measurements + base;
            const uint8_t* mk = ms->masks ? ms->masks + base : nullptr;
            const double inv_g = 1.0 / gains[f];
            // Natural column order first (contiguous, vectorised), then the
            // permutation: I / g in FP64 (by the reciprocal), rounded to
            // FP32, square root in FP32 (at most one ulp from rounding the
            // FP64 root).
            float a[256];
            for (int x = 0; x < N; ++x) a[x] = std::sqrt(std::fmax((float)(in[x] * inv_g), 0.0f));
            if (mk)
                for (int x = 0; x < N; ++x) a[x] = mk[x] == 0 ? -1.0f : a[x];
            float* o = reinterpret_cast<float*>(out);
            for (int t = 0; t < N; ++t) o[t] = a[column[t]];
        }));
    } else {
        FPM_TRY(upload_rows(ctx, p->meas.ptr, (long long)F * N, N * sizeof(float), s, [&](long long row, char* out) {
            const double* in = ms->measurements + ((size_t)(row / N) * N + natural_row(row % N)) * N;
            float* o = reinterpret_cast<float*>(out);
            for (int t = 0; t < N; ++t) o[t] = (float)in[column[t]];
        }));
        if (ms->masks) {
            FPM_TRY(p->masks.ensure(total));
            FPM_TRY(upload_rows(ctx, p->masks.ptr, (long long)F * N, N, s, [&](long long row, char* out) {
                const uint8_t* in = ms->masks + ((size_t)(row / N) * N + natural_row(row % N)) * N;
                for (int t = 0; t < N; ++t) out[t] = in[column[t]];
            }));
        }
    }
    if (md->background) {
        const long long bg_frames = p->background_stride ? F : 1;
        FPM_TRY(p->background.ensure((size_t)md->background_len * sizeof(float)));
        FPM_TRY(upload_rows(ctx, p->background.ptr, bg_frames * N, N * sizeof(float), s, [&](long long row, char* out) {
            const double* in = md->background + ((size_t)(row / N) * N + natural_row(row % N)) * N;
            float* o = reinterpret_cast<float*>(out);
            for (int t = 0; t < N; ++t) o[t] = (float)in[column[t]];
        }));
    }
    p->state_gains.resize(F);
    for (int f = 0; f < F; ++f) p->state_gains[f] = p->gains[f] > 0.0 ? p->gains[f] : 1.0;
    FPM_TRY(p->gains_d.ensure(F * sizeof(double)));
    FPM_TRY(upload_pageable(ctx, p->gains_d.ptr, p->state_gains.data(), F * sizeof(double), s));
    FPM_TRY(p->frame_params.ensure(sizeof(fpm::FrameParam) * F));
    FPM_TRY(upload_pageable(ctx, p->frame_params.ptr, p->params.data(), sizeof(fpm::FrameParam) * F, s));
    FPM_TRY(p->support_d.ensure(n2));
    FPM_TRY(upload_pageable(ctx, p->support_d.ptr, p->support.data(), n2, s));
    FPM_TRY(p->pupil_ref.ensure(n2 * sizeof(double2)));
    FPM_TRY(upload_pageable(ctx, p->pupil_ref.ptr, p->pupil.data(), n2 * sizeof(double2), s));
    std::vector<float2>& pf = p->pupil_f32;
    pf.resize(n2);
    for (size_t i = 0; i < n2; ++i) pf[i] = make_float2((float)p->pupil[2 * i], (float)p->pupil[2 * i + 1]);
    FPM_TRY(p->pupil_model.ensure(n2 * sizeof(float2)));
    FPM_TRY(upload_pageable(ctx, p->pupil_model.ptr, pf.data(), n2 * sizeof(float2), s));
    // Unit pupil: every value exactly 0 or 1 (FP32), the ones of each row on
    // one column interval. The single-CTA engine then reads the intervals
    // instead of the pupil; P * patch and U come out the same.
    std::vector<int2>& spans = p->pupil_spans;
    spans.assign(N, make_int2(0, -1));
    p->unit_pupil = true;
    for (int i = 0; i < N && p->unit_pupil; ++i) {
        int lo = N, hi = -1, ones = 0;
        for (int j = 0; j < N; ++j) {
            const float2 v = pf[(size_t)i * N + j];
            if (v.x == 0.f && v.y == 0.f) continue;
            if (v.x != 1.f || v.y != 0.f) {
                p->unit_pupil = false;
                break;
            }
            lo = std::min(lo, j);
            hi = std::max(hi, j);
            ++ones;
        }
        if (ones > 0 && ones != hi - lo + 1) p->unit_pupil = false;
        if (ones > 0) spans[i] = make_int2(lo, hi);
    }
    if (p->unit_pupil) {
        FPM_TRY(p->pupil_span.ensure(N * sizeof(int2)));
        FPM_TRY(upload_pageable(ctx, p->pupil_span.ptr, spans.data(), N * sizeof(int2), s));
    }
    return Status::ok();
}

Status create_problem(fpm_context* ctx, const fpm_model_desc* md, const fpm_measurement_desc* ms, fpm_problem** out) {
    FPM_TRY(validate_model(md));
    FPM_TRY(check_measurement_header(md, ms));
    std::vector<FrameScan> scans(ms->frames);
    HostPool::get().run(ms->frames, [&](long long f) { scan_frame(md, ms, (int)f, scans[f]); });
    FPM_TRY(check_scans(ms, scans.data()));
    std::unique_ptr<fpm_problem> p;
    FPM_TRY(prepare_problem(ctx, md, ms, scans.data(), p));
    cudaStream_t s = ctx->streams[0];
    FPM_TRY(upload_problem(ctx, p.get(), md, ms, s));
    FPM_CUDA(cudaStreamSynchronize(s));
    *out = p.release();
    return Status::ok();
}

// Many problems at once: every frame of every problem is scanned in one pass
// over the host threads, then all uploads are queued and synchronised once.
Status create_problems(fpm_context* ctx, int count, const fpm_model_desc* mds, const fpm_measurement_desc* mss,
                       std::vector<std::unique_ptr<fpm_problem>>& made) {
    std::vector<long long> first(count + 1, 0);
    for (int i = 0; i < count; ++i) {
        Status st = validate_model(&mds[i]);
        if (!st) st = check_measurement_header(&mds[i], &mss[i]);
        if (st) return Status::make(st.code, "problem %d: %s", i, st.message.c_str());
        first[i + 1] = first[i] + mss[i].frames;
    }
    std::vector<FrameScan> scans(first[count]);
    std::vector<int> owner(first[count]);
    for (int i = 0; i < count; ++i)
        for (long long k = first[i]; k < first[i + 1]; ++k) owner[k] = i;
    HostPool::get().run(first[count], [&](long long k) {
        const int i = owner[k];
        scan_frame(&mds[i], &mss[i], (int)(k - first[i]), scans[k]);
    });
    made.resize(count);
    for (int i = 0; i < count; ++i) {
        Status st = check_scans(&mss[i], scans.data() + first[i]);
        if (!st) st = prepare_problem(ctx, &mds[i], &mss[i], scans.data() + first[i], made[i]);
        if (st) return Status::make(st.code, "problem %d: %s", i, st.message.c_str());
    }
    cudaStream_t s = ctx->streams[0];
    for (int i = 0; i < count; ++i) FPM_TRY(upload_problem(ctx, made[i].get(), &mds[i], &mss[i], s));
    FPM_CUDA(cudaStreamSynchronize(s));
    return Status::ok();
}

// ------------------------------------------------------------------ runs

Status validate_params(const fpm_algorithm_params* a) {
    if (!a) return Status::make(FPM_ERR_INVALID_PARAMETER, "algorithm parameters are required");
    if (a->algorithm < FPM_ALG_AP || a->algorithm > FPM_ALG_ADAPTIVE_AP)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown algorithm %d", a->algorithm);
    if (a->iterations < 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "iterations must be non-negative");
    if (!std::isfinite(a->object_step) || a->object_step <= 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "object_step must be finite and positive");
    if (!std::isfinite(a->epsilon) || a->epsilon <= 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "epsilon must be finite and positive");
    if (a->batch_size <= 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "batch_size must be greater than zero");
    if (a->loss_type < 0 || a->loss_type > 3) return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown loss_type");
    if (a->schedule < 0 || a->schedule > 3) return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown schedule");
    if (a->algorithm == FPM_ALG_FPIE || a->algorithm == FPM_ALG_MPIE) {
        if (!std::isfinite(a->stability) || a->stability < 0.0 || a->stability > 1.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "stability must be finite and between zero and one");
    }
    if (a->algorithm == FPM_ALG_MPIE) {
        if (a->momentum_interval <= 0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "momentum_interval must be greater than zero");
        if (!std::isfinite(a->momentum_friction) || a->momentum_friction < 0.0 || a->momentum_friction >= 1.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "momentum_friction must be finite, at least zero, and less than one");
        if (!std::isfinite(a->momentum_feedback) || a->momentum_feedback < 0.0 || a->momentum_feedback > 1.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "momentum_feedback must be finite and between zero and one");
    }
    if (a->algorithm == FPM_ALG_EPRY) {
        if (!std::isfinite(a->pupil_step) || a->pupil_step < 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "pupil_step must be finite and non-negative");
        // Epry::validate (src/algorithms/epry.rs:206-236), for the recoveries requested.
        if (a->recover_frame_gains) {
            if (!std::isfinite(a->gain_step) || a->gain_step < 0.0 || a->gain_step > 1.0)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "gain_step must be finite and between zero and one");
            if (!std::isfinite(a->gain_min) || !std::isfinite(a->gain_max) || a->gain_min <= 0.0 ||
                a->gain_max <= a->gain_min)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "gain_bounds must be finite, positive, and strictly increasing");
        }
        if (a->recover_background) {
            if (!std::isfinite(a->background_step) || a->background_step < 0.0 || a->background_step > 1.0)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "background_step must be finite and between zero and one");
            if (!std::isfinite(a->background_min) || !std::isfinite(a->background_max) ||
                a->background_max <= a->background_min)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "background_bounds must be finite and strictly increasing");
        }
    }
    if (a->algorithm == FPM_ALG_ADAPTIVE_AP) {
        // AdaptiveAlternatingProjection::validate (src/algorithms/adaptive_alternating_projection.rs:350-403).
        if (a->iterations == 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "iterations must be greater than zero");
        if (!std::isfinite(a->progress_threshold) || a->progress_threshold < 0.0 || a->progress_threshold >= 1.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "progress_threshold must be finite, at least zero, and less than one");
        if (!std::isfinite(a->reduction_factor) || a->reduction_factor <= 0.0 || a->reduction_factor >= 1.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "reduction_factor must be finite, greater than zero, and less than one");
        if (!std::isfinite(a->minimum_object_step) || a->minimum_object_step <= 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "minimum_object_step must be finite and positive");
        if (a->minimum_object_step > a->object_step)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "minimum_object_step must not exceed initial_object_step");
    }
    if (a->algorithm == FPM_ALG_GD) {
        if (a->recover_pupil && (!std::isfinite(a->pupil_step) || a->pupil_step <= 0.0))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "pupil_step must be finite and positive");
        if (a->recover_pupil && a->poisson_truncation)
            return Status::make(FPM_ERR_UNSUPPORTED,
                                "gradient descent with both pupil recovery and Poisson truncation is not implemented "
                                "on the GB300 device path");
        // GradientDescent::validate (src/algorithms/gradient_descent.rs:319-383).
        if (!std::isfinite(a->object_tv_weight) || a->object_tv_weight < 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "object_tv_weight must be finite and non-negative");
        if (a->object_tv_weight > 0.0 && (!std::isfinite(a->object_tv_epsilon) || a->object_tv_epsilon <= 0.0))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "object_tv_epsilon must be finite and positive");
        if (!std::isfinite(a->pupil_smoothing_weight) || a->pupil_smoothing_weight < 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "pupil_smoothing_weight must be finite and non-negative");
        if (a->pupil_smoothing_weight > 0.0 && !a->recover_pupil)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "pupil_smoothing_weight requires recover_pupil");
        if ((a->object_tv_weight > 0.0 || a->pupil_smoothing_weight > 0.0) && a->poisson_truncation)
            return Status::make(FPM_ERR_UNSUPPORTED,
                                "gradient descent regularisers with Poisson truncation are not implemented on the "
                                "GB300 device path");
        if (a->recover_illumination) {
            const struct {
                double v;
                const char* name;
            } ill[3] = {{a->illumination_step, "illumination_step"},
                        {a->illumination_finite_difference, "illumination_finite_difference"},
                        {a->maximum_illumination_correction, "maximum_illumination_correction"}};
            for (const auto& v : ill)
                if (!std::isfinite(v.v) || v.v <= 0.0)
                    return Status::make(FPM_ERR_INVALID_PARAMETER, "%s must be finite and positive", v.name);
            if (a->recover_pupil || a->poisson_truncation)
                return Status::make(FPM_ERR_UNSUPPORTED,
                                    "illumination recovery with pupil recovery or Poisson truncation is not "
                                    "implemented on the GB300 device path");
        }
        if (a->poisson_truncation) {
            if (!std::isfinite(a->poisson_truncation_threshold) || a->poisson_truncation_threshold <= 0.0)
                return Status::make(FPM_ERR_INVALID_PARAMETER,
                                    "poisson_truncation_threshold must be finite and positive when provided");
            if (a->loss_type != FPM_LOSS_POISSON_NLL)
                return Status::make(FPM_ERR_INVALID_PARAMETER,
                                    "poisson_truncation_threshold requires Poisson negative log likelihood");
        }
    }
    return Status::ok();
}

// FrameSchedule::order_for_problem (src/reconstruction/schedule.rs:35-102).
std::vector<int> schedule_order(const fpm_problem* p, int schedule) {
    std::vector<int> order(p->frames);
    std::iota(order.begin(), order.end(), 0);
    if (schedule == FPM_SCHEDULE_SEQUENTIAL) return order;
    auto key = [](double v) {
        int64_t bits;
        std::memcpy(&bits, &v, sizeof bits);
        bits ^= (int64_t)(((uint64_t)(bits >> 63)) >> 1);
        return bits;
    };
    std::vector<std::pair<int64_t, int64_t>> keys(p->frames);
    for (int f = 0; f < p->frames; ++f) {
        if (schedule == FPM_SCHEDULE_SNR_WEIGHTED) {
            keys[f] = {key(-p->data_snr[f]), 0};
        } else {
            const double radius = std::hypot(p->kx[f], p->ky[f]);
            double angle = 0.0;
            if (schedule == FPM_SCHEDULE_SPIRAL_OUT) {
                angle = std::fmod(std::atan2(p->ky[f], p->kx[f]), 2.0 * M_PI);
                if (angle < 0.0) angle += 2.0 * M_PI;
            }
            keys[f] = {key(radius), key(angle)};
        }
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    return order;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// to the driver library); null when unavailable.
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled() {
    static const EncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (EncodeTiled) nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

// The stencil staging map of an M x MS complex64 object spectrum: viewed as
// [M rows][MS / 2 column pairs][4 floats], so every box starts at an aligned
// innermost coordinate (0) and a pair index (even column / 2); the box is
// (rows) x (n / 2 + 1 pairs) x 4, the (rows) x (n + 2) stencil slab.
bool encode_stencil_map(CUtensorMap* map, float2* object, int m, int n, int rows) {
    const EncodeTiled fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t ms = (cuuint64_t)(m + (m & 1));
    const cuuint64_t dims[3] = {4, ms / 2, (cuuint64_t)m};
    const cuuint64_t strides[2] = {16, ms * sizeof(float2)};
    const cuuint32_t box[3] = {4, (cuuint32_t)(n / 2 + 1), (cuuint32_t)rows};
    const cuuint32_t unit[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, object, dims, strides, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Bucket {
    int n, m;
    std::vector<fpm_problem*> problems;
    std::vector<int> indices;
    std::vector<const fpm_state_desc*> resume;  // per problem, or empty for a fresh start
};

// Pinned host storage for a run's tables: copies from it are asynchronous
// and do not wait for the work already queued on the run's stream (a copy
// from pageable memory would), and it lives as long as the run.
struct PinnedTables {
    std::vector<std::pair<char*, size_t>> blocks;  // (block, bytes used of kBlock or more)
    static constexpr size_t kBlock = size_t(1) << 20;
    size_t capacity = 0;
    ~PinnedTables() {
        for (auto& b : blocks) cudaFreeHost(b.first);
    }
    Status take(size_t bytes, char** at) {
        bytes = (bytes + 255) & ~size_t(255);
        if (blocks.empty() || blocks.back().second + bytes > capacity) {
            const size_t size = std::max(kBlock, bytes);
            char* block = nullptr;
            FPM_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&block), size, cudaHostAllocDefault));
            blocks.emplace_back(block, 0);
            capacity = size;
        }
        *at = blocks.back().first + blocks.back().second;
        blocks.back().second += bytes;
        return Status::ok();
    }
};

template <class T>
Status upload_array(fpm_context* ctx, DeviceBuffer& buf, const std::vector<T>& v, cudaStream_t s) {
    FPM_TRY(buf.ensure(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty()) FPM_TRY(upload_pageable(ctx, buf.ptr, v.data(), sizeof(T) * v.size(), s));
    return Status::ok();
}

// A run's table: staged in the run's own pinned storage and copied on its stream.
template <class T>
Status upload_table(PinnedTables& tables, DeviceBuffer& buf, const std::vector<T>& v, cudaStream_t s) {
    FPM_TRY(buf.ensure(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (v.empty()) return Status::ok();
    char* at = nullptr;
    FPM_TRY(tables.take(sizeof(T) * v.size(), &at));
    std::memcpy(at, v.data(), sizeof(T) * v.size());
    FPM_CUDA(cudaMemcpyAsync(buf.ptr, at, sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return Status::ok();
}

// A problem's per-run buffers: bound to the stream of the run that uses them.
std::vector<DeviceBuffer*> run_buffers(fpm_problem* p) {
    return {&p->object,     &p->pupil_state,   &p->partials,       &p->counter,    &p->status,
            &p->scratch64,  &p->velocity,      &p->anchor,         &p->order,      &p->gradient,
            &p->pupil_gradient, &p->tv_scratch, &p->pupil_scratch, &p->ill_params, &p->ill_start,
            &p->ill_offset, &p->ill_correction, &p->ill_partials, &p->object_err, &p->gradient_err,
            &p->gain_state, &p->bg_state, &p->bg_natural};
}

struct BucketRun {
    PinnedTables tables;         // host sources of the run's table uploads
    DeviceBuffer field_scratch;  // single-CTA engine: per-CTA field scratch
    DeviceBuffer recovery;       // EPRY gain / background recovery: per-tile state pointers
    DeviceBuffer tmaps;  // per tile: the object spectrum's tensor map for TMA stencil staging
    DeviceBuffer tiles, init, gauge, scratch_ptrs, object_ptrs, anchor_ptrs, velocity_ptrs, avg, init_partial,
        tv_ptrs, tv_objects, tv_table, smooth_table, ill_tiles, ill_tasks, ill_fields, ill_valid, ill_ptrs;
    std::vector<cudaEvent_t> events;  // (start, end) pairs around engine launches
    cudaEvent_t first = nullptr, last = nullptr;
    int launches = 0;
    double bytes = 0.0;
    // A run is prepared (host work, buffers, uploads of its tables) and
    // launched (device work only). Captured run plans do the two apart: the
    // preparation once, the launch inside a CUDA graph capture.
    bool prepare = true, launch = true;
    bool captured = false;  // launched inside a stream capture: timing events become graph nodes
    cudaError_t record(cudaEvent_t e, cudaStream_t s) const {
        // Inside a capture a plain record only orders streams; an external
        // record is a node that records the event at each replay.
        return captured ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
    }
    ~BucketRun() {
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        if (first) cudaEventDestroy(first);
        if (last) cudaEventDestroy(last);
    }
};

int engine_grid_slot(int n) { return n == 32 ? 0 : n == 64 ? 1 : n == 128 ? 2 : n == 256 ? 3 : -1; }

// Whether a launch of `tiles` tiles of size n takes the single-CTA engine
// (alg: its family; `eligible`: measurements and options it takes). AUTO
// picks it once the launch holds at least two thirds of the CTAs that fit
// at once: a lone tile then runs about seven times longer on one CTA than
// on a 16-CTA cluster, while a full device of single CTAs has the higher
// throughput.
Status single_cta_engine(const fpm_context* ctx, int n, int alg, bool eligible, int tiles, bool* single,
                         int* resident) {
    *single = false;
    *resident = 0;
    const int k = engine_grid_slot(n);
    if (k < 0 || ctx->engine_shape[k] == FPM_ENGINE_CLUSTER || !eligible || !fpm::engine_l2_supported(n, alg))
        return Status::ok();
    FPM_CUDA(fpm::engine_l2_max_active_ctas(n, resident));
    *single = ctx->engine_shape[k] == FPM_ENGINE_SINGLE_CTA || 3 * tiles >= 2 * *resident;
    return Status::ok();
}

// Clusters of an engine launch over `tiles` tiles of size n.
int engine_clusters(const fpm_context* ctx, int n, int tiles) {
    const int k = engine_grid_slot(n);
    const int g = k >= 0 ? ctx->engine_grid[k] : 0;
    return g > 0 && g < tiles ? g : tiles;
}

// The frame-engine family of an algorithm's parameters.
int engine_family(const fpm_algorithm_params* a) {
    switch (a->algorithm) {
        case FPM_ALG_AP: return fpm::kAlgLocal;
        case FPM_ALG_ADAPTIVE_AP: return fpm::kAlgLocalAdaptive;
        case FPM_ALG_FPIE:
        case FPM_ALG_MPIE: return fpm::kAlgRpie;
        case FPM_ALG_EPRY:
            if (a->recover_frame_gains || a->recover_background)
                return a->recover_pupil ? fpm::kAlgEpryCal : fpm::kAlgGlobalCal;
            return a->recover_pupil ? fpm::kAlgEpry : fpm::kAlgGlobal;
        default:
            return a->recover_pupil       ? fpm::kAlgGradientPupil
                   : a->poisson_truncation ? fpm::kAlgGradientTruncated
                                           : fpm::kAlgGradient;
    }
}

Status run_bucket(fpm_context* ctx, Bucket& b, const fpm_algorithm_params* a, cudaStream_t s, BucketRun& br) {
    const int N = b.n, M = b.m, count = (int)b.problems.size();
    const int C = fpm::engine_ctas(N);
    const long long ms = M + (M & 1);
    const bool mpie = a->algorithm == FPM_ALG_MPIE;
    const bool epry = a->algorithm == FPM_ALG_EPRY;
    const bool gd_pupil = a->algorithm == FPM_ALG_GD && a->recover_pupil;
    // Pupil-recovering runs canonicalise the object/pupil gauge at the start
    // and after every iteration (Runner::run, src/reconstruction/runner.rs:122,220).
    const bool canonical = (epry && a->recover_pupil) || gd_pupil;
    const bool gd_batched = a->algorithm == FPM_ALG_GD && a->batch_size > 1;
    // Kahan summation of the frame updates into the object (or the mini-batch gradient).
    const bool compensated = a->compensated_accumulation != 0;
    // GD regularisers run between per-batch engine launches.
    const bool tv = a->algorithm == FPM_ALG_GD && a->object_tv_weight > 0.0;
    const bool smoothing = gd_pupil && a->pupil_smoothing_weight > 0.0;
    // Illumination recovery: a finite-difference gradient launch before and a
    // correction update after each GD batch's engine launch.
    // EPRY frame-gain / background recovery: state gains and backgrounds on the device.
    const bool recover_gb = epry && (a->recover_frame_gains || a->recover_background);
    const bool illum = a->algorithm == FPM_ALG_GD && a->recover_illumination;
    const bool regularised = tv || smoothing || illum;
    const int iters = a->iterations;
    const bool resumed = !b.resume.empty();
    const int it0 = resumed ? b.resume[0]->completed_iterations : 0;
    std::vector<fpm::TileDesc> tiles(count);
    // 256-point tiles stage their stencils with TMA, through one tensor map per tile.
    const bool tma = N == 256;
    std::vector<CUtensorMap> maps(tma ? count : 0);
    if (tma) {
        br.tmaps.bind(ctx->pool, s);
        FPM_TRY(br.tmaps.ensure(sizeof(CUtensorMap) * (size_t)count));
    }
    std::vector<fpm::InitTile> inits(count);
    std::vector<fpm::TileRecovery> recovery(count);
    std::vector<fpm::GaugeTile> gauges(count);
    std::vector<fpm::IlluminationTile> ill_tiles(illum ? count : 0);
    std::vector<double2*> scratch(count);
    std::vector<float2*> objects(count), anchors(count), velocities(count);
    double max_pupil_power = 0.0;
    for (int t = 0; t < count; ++t) {
        fpm_problem* p = b.problems[t];
        const size_t n2 = (size_t)N * N;
        for (DeviceBuffer* buf : run_buffers(p)) buf->bind(ctx->pool, s);
        FPM_TRY(p->object.ensure(sizeof(float2) * (size_t)M * ms));
        FPM_TRY(p->pupil_state.ensure(sizeof(float2) * n2));
        FPM_TRY(p->partials.ensure(sizeof(double) * std::max(iters, 1) * C));
        FPM_TRY(p->counter.ensure(sizeof(int)));
        FPM_TRY(p->status.ensure(sizeof(int)));
        FPM_TRY(p->scratch64.ensure(sizeof(double2) * (size_t)M * M));
        if (gd_batched) {
            FPM_TRY(p->gradient.ensure(sizeof(float2) * (size_t)M * ms));
            if (br.launch) FPM_CUDA(cudaMemsetAsync(p->gradient.ptr, 0, sizeof(float2) * (size_t)M * ms, s));
        }
        if (gd_pupil) {
            FPM_TRY(p->pupil_gradient.ensure(sizeof(float2) * n2));
            if (br.launch) FPM_CUDA(cudaMemsetAsync(p->pupil_gradient.ptr, 0, sizeof(float2) * n2, s));
        }
        if (compensated) {
            DeviceBuffer& e = gd_batched ? p->gradient_err : p->object_err;
            FPM_TRY(e.ensure(sizeof(float2) * (size_t)M * ms));
            if (br.launch) FPM_CUDA(cudaMemsetAsync(e.ptr, 0, sizeof(float2) * (size_t)M * ms, s));
        }
        if (tv) FPM_TRY(p->tv_scratch.ensure(sizeof(double2) * (size_t)M * M));
        if (smoothing) FPM_TRY(p->pupil_scratch.ensure(sizeof(float2) * n2));
        if (mpie) {
            FPM_TRY(p->velocity.ensure(sizeof(float2) * (size_t)M * ms));
            FPM_TRY(p->anchor.ensure(sizeof(float2) * (size_t)M * ms));
        }
        if (br.launch) FPM_CUDA(cudaMemsetAsync(p->status.ptr, 0, sizeof(int), s));
        if (recover_gb) {
            // State gains start at the model's; state backgrounds at the
            // model's (one shared image or one per frame) or zero.
            const int F = p->frames;
            const size_t n2f = (size_t)N * N;
            FPM_TRY(p->gain_state.ensure(sizeof(double) * F));
            FPM_TRY(p->bg_state.ensure(sizeof(float) * n2f * F));
            if (br.launch) {
                FPM_CUDA(cudaMemcpyAsync(p->gain_state.ptr, p->gains_d.ptr, sizeof(double) * F, cudaMemcpyDeviceToDevice, s));
                if (!p->has_background) {
                    FPM_CUDA(cudaMemsetAsync(p->bg_state.ptr, 0, sizeof(float) * n2f * F, s));
                } else if (p->background_stride == 0) {
                    for (int f = 0; f < F; ++f)
                        FPM_CUDA(cudaMemcpyAsync(p->bg_state.as<float>() + (size_t)f * n2f, p->background.ptr,
                                                 sizeof(float) * n2f, cudaMemcpyDeviceToDevice, s));
                } else {
                    FPM_CUDA(cudaMemcpyAsync(p->bg_state.ptr, p->background.ptr, sizeof(float) * n2f * F,
                                             cudaMemcpyDeviceToDevice, s));
                }
            }
        }
        p->it0 = it0;
        p->resume_objectives.clear();
        if (resumed) {
            // Restore the saved state: complex128 host arrays through scratch64
            // into the complex64 state (stream-ordered reuse of scratch64).
            const fpm_state_desc* r = b.resume[t];
            p->resume_objectives.assign(r->objectives, r->objectives + it0);
            p->host_counter = mpie ? r->momentum_counter : 0;
            FPM_CUDA(cudaMemcpyAsync(p->counter.ptr, &p->host_counter, sizeof(int), cudaMemcpyHostToDevice, s));
            double2* wide = p->scratch64.as<double2>();
            FPM_CUDA(cudaMemcpyAsync(wide, r->pupil, sizeof(double2) * n2, cudaMemcpyHostToDevice, s));
            FPM_CUDA(fpm::launch_narrow(wide, N, N, p->pupil_state.as<float2>(), N, s));
            const struct {
                const double* src;
                DeviceBuffer* dst;
            } grids[3] = {{r->object_spectrum, &p->object}, {r->velocity, &p->velocity}, {r->anchor, &p->anchor}};
            for (int g = 0; g < (mpie ? 3 : 1); ++g) {
                FPM_CUDA(cudaMemcpyAsync(wide, grids[g].src, sizeof(double2) * (size_t)M * M, cudaMemcpyHostToDevice, s));
                FPM_CUDA(fpm::launch_narrow(wide, M, M, grids[g].dst->as<float2>(), ms, s));
            }
            br.launches += mpie ? 4 : 2;
        } else if (br.launch) {
            FPM_CUDA(cudaMemsetAsync(p->counter.ptr, 0, sizeof(int), s));
            FPM_CUDA(cudaMemcpyAsync(p->pupil_state.ptr, p->pupil_model.ptr, sizeof(float2) * n2, cudaMemcpyDeviceToDevice, s));
        }
        const int* order_dev = nullptr;
        if (a->schedule != FPM_SCHEDULE_SEQUENTIAL) {
            if (br.prepare) FPM_TRY(upload_table(br.tables, p->order, schedule_order(p, a->schedule), s));
            order_dev = p->order.as<int>();
        }
        // max(max |P|^2, eps) of the compiled pupil, FP64.
        double mp = 0.0;
        for (size_t i = 0; i < n2; ++i)
            mp = std::max(mp, p->pupil[2 * i] * p->pupil[2 * i] + p->pupil[2 * i + 1] * p->pupil[2 * i + 1]);
        mp = std::max(mp, a->epsilon);
        max_pupil_power = mp;
        fpm::TileDesc& T = tiles[t];
        T.object = p->object.as<float2>();
        T.pupil = p->pupil_state.as<float2>();
        T.support = p->support_d.as<uint8_t>();
        T.meas = p->meas.as<float>();
        T.amplitude = p->amplitude ? 1 : 0;
        T.weight_sum = p->weight_sum;
        // Centred rows holding a non-zero (FP32) pupil value.
        T.row_lo = N;
        T.row_hi = -1;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const float2 v = p->pupil_f32[(size_t)i * N + j];
                if (v.x != 0.f || v.y != 0.f) {
                    T.row_lo = std::min(T.row_lo, i);
                    T.row_hi = std::max(T.row_hi, i);
                }
            }
        // A resumed run's pupil comes from its checkpoint, not the compiled model.
        T.pupil_span = p->unit_pupil && !resumed ? p->pupil_span.as<int2>() : nullptr;
        T.masks = p->has_masks && !p->amplitude ? p->masks.as<uint8_t>() : nullptr;
        T.background = p->has_background ? p->background.as<float>() : nullptr;
        T.background_stride = p->background_stride;
        T.params = p->frame_params.as<fpm::FrameParam>();
        T.omap = nullptr;
        if (tma && encode_stencil_map(&maps[t], p->object.as<float2>(), M, N, fpm::engine_rows(N) + 1))
            T.omap = br.tmaps.as<CUtensorMap>() + t;
        T.order = order_dev;
        if (illum) {
            // The run's own frame constants follow the recovered offsets; the
            // problem's resident ones stay as compiled.
            const int F = p->frames;
            FPM_TRY(p->ill_params.ensure(sizeof(fpm::FrameParam) * F));
            FPM_TRY(p->ill_correction.ensure(sizeof(double) * 2 * F));
            const double* saved = resumed ? b.resume[t]->illumination_corrections : nullptr;
            if (!br.launch) {
                // Prepared only: the run copies its frame constants when launched.
            } else if (saved) {
                // A checkpoint's corrections and the stencils they imply.
                std::vector<fpm::FrameParam> prm(p->params);
                for (int f = 0; f < F; ++f)
                    if (!fpm::offset_frame_param(p->start_row[f], p->start_col[f], p->off_row[f] + saved[2 * f],
                                                 p->off_col[f] + saved[2 * f + 1], N, M, prm[f]))
                        return Status::make(FPM_ERR_INVALID_PARAMETER,
                                            "checkpoint illumination correction of source %d moves its crop outside "
                                            "the reconstruction grid", f);
                FPM_TRY(upload_table(br.tables, p->ill_params, prm, s));
                FPM_CUDA(cudaMemcpyAsync(p->ill_correction.ptr, saved, sizeof(double) * 2 * F,
                                         cudaMemcpyHostToDevice, s));
            } else {
                FPM_CUDA(cudaMemcpyAsync(p->ill_params.ptr, p->frame_params.ptr, sizeof(fpm::FrameParam) * F,
                                         cudaMemcpyDeviceToDevice, s));
                FPM_CUDA(cudaMemsetAsync(p->ill_correction.ptr, 0, sizeof(double) * 2 * F, s));
            }
            std::vector<long long> start(2 * (size_t)F);
            std::vector<double> offset(2 * (size_t)F);
            for (int f = 0; f < F; ++f) {
                start[2 * f] = p->start_row[f];
                start[2 * f + 1] = p->start_col[f];
                offset[2 * f] = p->off_row[f];
                offset[2 * f + 1] = p->off_col[f];
            }
            if (br.prepare) {
                FPM_TRY(upload_table(br.tables, p->ill_start, start, s));
                FPM_TRY(upload_table(br.tables, p->ill_offset, offset, s));
            }
            FPM_TRY(p->ill_partials.ensure(sizeof(double) * 4 * fpm::kIlluminationBlocks * (size_t)F));
            T.params = p->ill_params.as<fpm::FrameParam>();
            fpm::IlluminationTile& L = ill_tiles[t];
            L.object = T.object;
            L.pupil = T.pupil;
            L.meas = T.meas;
            L.masks = T.masks;
            L.background = T.background;
            L.background_stride = T.background_stride;
            L.params = p->ill_params.as<fpm::FrameParam>();
            L.order = order_dev;
            L.start = p->ill_start.as<long long>();
            L.offset = p->ill_offset.as<double>();
            L.correction = p->ill_correction.as<double>();
            L.partials = p->ill_partials.as<double>();
            L.status = p->status.as<int>();
            L.M = M;
            L.frame_count = F;
            L.amplitude = T.amplitude;
        }
        T.velocity = mpie ? p->velocity.as<float2>() : nullptr;
        T.anchor = mpie ? p->anchor.as<float2>() : nullptr;
        T.gradient = gd_batched ? p->gradient.as<float2>() : nullptr;
        T.object_err = compensated && !gd_batched ? p->object_err.as<float2>() : nullptr;
        T.gradient_err = compensated && gd_batched ? p->gradient_err.as<float2>() : nullptr;
        T.pupil_gradient = gd_pupil ? p->pupil_gradient.as<float2>() : nullptr;
        recovery[t] = {recover_gb ? p->gain_state.as<double>() : nullptr, recover_gb ? p->bg_state.as<float>() : nullptr};
        T.partials = p->partials.as<double>();
        T.counter = p->counter.as<int>();
        T.status = p->status.as<int>();
        T.M = M;
        T.frame_count = p->frames;
        T.max_pupil_power = max_pupil_power;
        fpm::InitTile& I = inits[t];
        I.meas = T.meas;
        I.amplitude = T.amplitude;
        I.masks = T.masks;
        I.background = T.background;
        I.background_stride = T.background_stride;
        I.params = T.params;
        I.scratch = p->scratch64.as<double2>();
        I.status = T.status;
        I.frames_count = p->frames;
        fpm::GaugeTile& G = gauges[t];
        G.object = T.object;
        G.pupil = T.pupil;
        G.reference = p->pupil_ref.as<double2>();
        G.support = T.support;
        G.status = T.status;
        G.row_exact = p->row_exact ? 1 : 0;
        G.col_exact = p->col_exact ? 1 : 0;
        scratch[t] = p->scratch64.as<double2>();
        objects[t] = T.object;
        anchors[t] = T.anchor;
        velocities[t] = T.velocity;
        // Algorithmic bytes of the engine for this tile (counted when prepared).
        if (!br.prepare) continue;
        double frame_bytes = 0.0;
        int effective = 0;
        for (int f = 0; f < p->frames; ++f) {
            if (p->params[f].weight == 0.f) continue;
            ++effective;
            frame_bytes += 16.0 * p->stencil_cells[f] + 4.0 * (double)n2 + (p->has_masks && !p->amplitude ? (double)n2 : 0.0) +
                           (canonical ? 16.0 * (double)n2 : 0.0);
        }
        br.bytes += frame_bytes * iters;
        if (compensated) {
            // The error term's read and write beside every stencil update.
            double err = 0.0;
            for (int f = 0; f < p->frames; ++f)
                if (p->params[f].weight != 0.f) err += 16.0 * p->stencil_cells[f];
            br.bytes += err * iters;
        }
        if (a->algorithm == FPM_ALG_GD && a->poisson_truncation) {
            // Forward-only statistics pass: stencil read and measurement per frame,
            // and |O|^2 of the grid per batch.
            double fwd = 0.0;
            for (int f = 0; f < p->frames; ++f)
                if (p->params[f].weight != 0.f) fwd += 8.0 * p->stencil_cells[f] + 4.0 * (double)n2;
            const long long batches = (p->frames + a->batch_size - 1) / a->batch_size;
            br.bytes += (fwd + 8.0 * (double)M * (double)ms * (double)batches) * iters;
        }
        if (gd_batched) {
            // Gradient read-modify-write per frame; object and gradient pass per batch.
            double stencil = 0.0;
            for (int f = 0; f < p->frames; ++f)
                if (p->params[f].weight != 0.f) stencil += 16.0 * p->stencil_cells[f];
            const long long batches = (p->frames + a->batch_size - 1) / a->batch_size;
            br.bytes += (stencil + 32.0 * (double)M * (double)ms * (double)batches) * iters;
        }
        if (mpie && a->momentum_interval > 0)
            br.bytes += 48.0 * (double)M * (double)M * (double)((long long)effective * iters / a->momentum_interval);
    }
    for (DeviceBuffer* buf : {&br.tiles, &br.init, &br.gauge, &br.scratch_ptrs, &br.object_ptrs, &br.anchor_ptrs,
                              &br.velocity_ptrs, &br.avg, &br.init_partial, &br.tv_ptrs, &br.tv_objects,
                              &br.tv_table, &br.smooth_table, &br.ill_tiles, &br.ill_tasks, &br.ill_fields,
                              &br.ill_valid, &br.ill_ptrs, &br.recovery})
        buf->bind(ctx->pool, s);
    if (!br.first) FPM_CUDA(cudaEventCreate(&br.first));
    if (!br.last) FPM_CUDA(cudaEventCreate(&br.last));
    if (br.prepare) {
        if (tma) FPM_TRY(upload_table(br.tables, br.tmaps, maps, s));
        FPM_TRY(upload_table(br.tables, br.tiles, tiles, s));
        FPM_TRY(upload_table(br.tables, br.init, inits, s));
        FPM_TRY(upload_table(br.tables, br.gauge, gauges, s));
        FPM_TRY(upload_table(br.tables, br.scratch_ptrs, scratch, s));
        FPM_TRY(upload_table(br.tables, br.object_ptrs, objects, s));
        FPM_TRY(upload_table(br.tables, br.anchor_ptrs, anchors, s));
        FPM_TRY(upload_table(br.tables, br.velocity_ptrs, velocities, s));
        // The line FFT plans of both grids exist before any launch (a plan's
        // creation synchronises, which a graph capture cannot).
        FftPlan* plan = nullptr;
        FPM_TRY(get_plan(ctx, M, plan));
        FPM_TRY(get_plan(ctx, N, plan));
    }
    if (br.launch) FPM_CUDA(br.record(br.first, s));

    // Initial object: mean amplitude, upsample, forward FFT (FP64), fftshift;
    // one launch pair for all tiles of the bucket. A resumed run has restored
    // its state above. Pupil-recovering runs canonicalise either way.
    FPM_TRY(br.avg.ensure(sizeof(double) * (size_t)N * N * count));
    FPM_TRY(br.init_partial.ensure(sizeof(double) * 2 * (size_t)fpm::init_chunks(N) * count));
    if (!resumed && br.launch) {
        FPM_CUDA(fpm::launch_init_mean(N, M, br.init.as<fpm::InitTile>(), count, br.avg.as<double>(),
                                       br.init_partial.as<double>(), s));
        br.launches += 2;
        FPM_TRY(fft2_device(ctx, br.scratch_ptrs.as<double2*>(), count, M, M, false, s));
        FPM_CUDA(fpm::launch_shift_to_state(br.scratch_ptrs.as<double2*>(), br.object_ptrs.as<float2*>(),
                                            mpie ? br.anchor_ptrs.as<float2*>() : nullptr,
                                            mpie ? br.velocity_ptrs.as<float2*>() : nullptr, count, M, s));
        br.launches += 3;
    }
    if (canonical && br.launch) {
        FPM_CUDA(fpm::launch_gauge(br.gauge.as<fpm::GaugeTile>(), count, N, M, s));
        br.launches += 1;
    }

    fpm::EngineParams ep{};
    ep.tiles = br.tiles.as<fpm::TileDesc>();
    ep.tile_count = count;
    ep.alg = engine_family(a);
    ep.alpha = a->stability;
    ep.eps = a->epsilon;
    ep.object_step = a->object_step;
    ep.pupil_step = a->pupil_step;
    // With pupil smoothing the support is imposed after the smoothing step.
    ep.constrain_pupil = a->constrain_pupil_support && !smoothing ? 1 : 0;
    ep.momentum = mpie ? 1 : 0;
    ep.interval = a->momentum_interval;
    ep.friction = (float)a->momentum_friction;
    ep.feedback = (float)a->momentum_feedback;
    // The adaptive controller's objective is always amplitude MSE.
    ep.loss = a->algorithm == FPM_ALG_ADAPTIVE_AP ? FPM_LOSS_AMPLITUDE_MSE : a->loss_type;
    ep.progress_threshold = a->progress_threshold;
    ep.reduction_factor = a->reduction_factor;
    ep.minimum_step = a->minimum_object_step;
    ep.gd_batch = a->algorithm == FPM_ALG_GD ? a->batch_size : 1;
    ep.trunc_threshold = a->algorithm == FPM_ALG_GD && a->poisson_truncation ? (float)a->poisson_truncation_threshold : 0.f;
    if (recover_gb) {
        if (br.prepare) FPM_TRY(upload_table(br.tables, br.recovery, recovery, s));
        ep.recovery = br.recovery.as<fpm::TileRecovery>();
    }
    ep.recover_gains = recover_gb && a->recover_frame_gains ? 1 : 0;
    ep.recover_background = recover_gb && a->recover_background ? 1 : 0;
    ep.gain_step = a->gain_step;
    ep.gain_min = a->gain_min;
    ep.gain_max = a->gain_max;
    ep.background_step = a->background_step;
    ep.background_min = a->background_min;
    ep.background_max = a->background_max;
    // The single-CTA engine takes 256-point tiles of the fixed-pupil
    // projection families with amplitude-form measurements and plain
    // accumulation; other runs use the cluster engine.
    bool all_amplitude = true;
    for (fpm_problem* p : b.problems) all_amplitude = all_amplitude && p->amplitude;
    bool single = false;
    int resident = 0;
    FPM_TRY(single_cta_engine(ctx, N, ep.alg, all_amplitude && !compensated && !regularised && !recover_gb, count,
                              &single, &resident));
    int units = engine_clusters(ctx, N, count);
    if (single) {
        const int want = ctx->engine_ctas[engine_grid_slot(N)];
        units = std::max(1, std::min(count, want > 0 ? want : resident));
        br.field_scratch.bind(ctx->pool, s);
        FPM_TRY(br.field_scratch.ensure(fpm::engine_l2_scratch_bytes(N) * (size_t)units));
        ep.field_scratch = br.field_scratch.as<float2>();
        ep.unit_pupils = 1;
        for (const fpm::TileDesc& T : tiles) ep.unit_pupils &= T.pupil_span != nullptr ? 1 : 0;
    }
    auto engine = [&](int it0, int it1) -> Status {
        cudaEvent_t e0, e1;
        FPM_CUDA(cudaEventCreate(&e0));
        FPM_CUDA(cudaEventCreate(&e1));
        br.events.push_back(e0);
        br.events.push_back(e1);
        ep.it_begin = it0;
        ep.it_end = it1;
        FPM_CUDA(br.record(e0, s));
        if (single) FPM_CUDA(fpm::launch_engine_l2(N, ep, units, s));
        else FPM_CUDA(fpm::launch_engine(N, ep, units, s));
        FPM_CUDA(br.record(e1, s));
        br.launches += 1;
        return Status::ok();
    };
    if (iters > it0 && regularised) {
        // One launch per GD batch (order positions [b B, (b + 1) B)), then the
        // regularisers scaled by each tile's batch share of its frames; a tile
        // whose frames are exhausted keeps its state.
        const int B = a->batch_size;
        int fmax = 0;
        for (fpm_problem* p : b.problems) fmax = std::max(fmax, p->frames);
        const int nb = (fmax + B - 1) / B;
        std::vector<fpm::RegularTile> tv_table, smooth_table;
        std::vector<double2*> tv_ptrs(count);
        std::vector<float2*> tv_objects((size_t)nb * count);
        for (int k = 0; k < nb; ++k)
            for (int t = 0; t < count; ++t) {
                fpm_problem* p = b.problems[t];
                const int in_batch = std::max(0, std::min((k + 1) * B, p->frames) - k * B);
                const double fraction = (double)in_batch / (double)p->frames;
                fpm::RegularTile r{};
                r.src = p->scratch64.as<double2>();
                r.dst = tv ? p->tv_scratch.as<double2>() : nullptr;
                r.pupil = p->pupil_state.as<float2>();
                r.pupil_scratch = smoothing ? p->pupil_scratch.as<float2>() : nullptr;
                r.support = p->support_d.as<uint8_t>();
                r.status = p->status.as<int>();
                r.weight = a->object_tv_weight * fraction;
                tv_table.push_back(r);
                r.weight = a->pupil_smoothing_weight * fraction;
                smooth_table.push_back(r);
                tv_objects[(size_t)k * count + t] = in_batch > 0 ? p->object.as<float2>() : nullptr;
                if (k == 0) tv_ptrs[t] = tv ? p->tv_scratch.as<double2>() : nullptr;
            }
        if (br.prepare) {
            FPM_TRY(upload_table(br.tables, br.tv_table, tv_table, s));
            FPM_TRY(upload_table(br.tables, br.smooth_table, smooth_table, s));
            FPM_TRY(upload_table(br.tables, br.tv_ptrs, tv_ptrs, s));
            FPM_TRY(upload_table(br.tables, br.tv_objects, tv_objects, s));
        }
        // Illumination tasks of batch k: [k * batch_tasks, (k + 1) * batch_tasks),
        // evaluated in chunks of at most `chunk` tasks (5 FP64 N x N fields
        // each, about 256 MB at most). Positions past the longest tile never
        // hold a frame, so a batch larger than every tile needs only fmax
        // tasks per tile.
        fpm::IlluminationParams ip{};
        const int task_b = std::min(B, fmax);
        const int batch_tasks = count * task_b;
        const size_t field_bytes = sizeof(double2) * 5 * (size_t)N * N;
        const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)batch_tasks, (256u << 20) / field_bytes));
        if (illum) {
            std::vector<fpm::IlluminationTask> tasks;
            tasks.reserve((size_t)nb * batch_tasks);
            for (int k = 0; k < nb; ++k)
                for (int t = 0; t < count; ++t)
                    for (int j = 0; j < task_b; ++j) tasks.push_back({t, k * B + j});
            FPM_TRY(br.ill_fields.ensure(field_bytes * chunk));
            FPM_TRY(br.ill_valid.ensure(sizeof(int) * 5 * (size_t)chunk));
            if (br.prepare) {
                FPM_TRY(upload_table(br.tables, br.ill_tiles, ill_tiles, s));
                FPM_TRY(upload_table(br.tables, br.ill_tasks, tasks, s));
                std::vector<double2*> ptrs((size_t)5 * chunk);
                for (size_t i = 0; i < ptrs.size(); ++i) ptrs[i] = br.ill_fields.as<double2>() + i * (size_t)N * N;
                FPM_TRY(upload_table(br.tables, br.ill_ptrs, ptrs, s));
            }
            ip.tiles = br.ill_tiles.as<fpm::IlluminationTile>();
            ip.fields = br.ill_fields.as<double2>();
            ip.valid = br.ill_valid.as<int>();
            ip.distance = a->illumination_finite_difference;
            ip.epsilon = a->epsilon;
            ip.loss = a->loss_type;
            ip.n = N;
        }
        for (int it = it0; it < iters && br.launch; ++it) {
            for (int k = 0; k < nb; ++k) {
                ep.frame_begin = k * B;
                ep.frame_end = (k + 1) * B;
                ep.accumulate = k > 0 ? 1 : 0;
                const fpm::IlluminationTask* batch = br.ill_tasks.as<fpm::IlluminationTask>() + (size_t)k * batch_tasks;
                // illumination_gradient from the batch-start object and pupil
                // (src/algorithms/gradient_descent.rs:590-613), FP64.
                for (int c0 = 0; illum && c0 < batch_tasks; c0 += chunk) {
                    const int n_tasks = std::min(chunk, batch_tasks - c0);
                    ip.tasks = batch + c0;
                    FPM_CUDA(fpm::launch_illumination_fields(ip, n_tasks, s));
                    FPM_TRY(fft2_device(ctx, br.ill_ptrs.as<double2*>(), 5 * n_tasks, N, N, true, s));
                    FPM_CUDA(fpm::launch_illumination_reduce(ip, n_tasks, s));
                    br.launches += 4;
                }
                FPM_TRY(engine(it, it + 1));
                if (illum) {
                    FPM_CUDA(fpm::launch_illumination_update(br.ill_tiles.as<fpm::IlluminationTile>(), batch,
                                                             batch_tasks, N, a->illumination_step,
                                                             a->maximum_illumination_correction, a->epsilon, s));
                    br.launches += 1;
                }
                if (tv) {
                    // apply_object_tv (src/algorithms/gradient_descent.rs:1125-1165) in FP64.
                    FPM_CUDA(fpm::launch_state_to_natural(reinterpret_cast<const float2* const*>(br.object_ptrs.ptr),
                                                          br.scratch_ptrs.as<double2*>(), count, M, s));
                    FPM_TRY(fft2_device(ctx, br.scratch_ptrs.as<double2*>(), count, M, M, true, s));
                    FPM_CUDA(fpm::launch_object_tv(br.tv_table.as<fpm::RegularTile>() + (size_t)k * count, count, M,
                                                   a->object_tv_epsilon, s));
                    FPM_TRY(fft2_device(ctx, br.tv_ptrs.as<double2*>(), count, M, M, false, s));
                    FPM_CUDA(fpm::launch_shift_to_state(br.tv_ptrs.as<double2*>(),
                                                        br.tv_objects.as<float2*>() + (size_t)k * count, nullptr,
                                                        nullptr, count, M, s));
                    br.launches += 7;
                }
                if (smoothing) {
                    FPM_CUDA(fpm::launch_pupil_smoothing(br.smooth_table.as<fpm::RegularTile>() + (size_t)k * count,
                                                         count, N, a->constrain_pupil_support ? 1 : 0, s));
                    br.launches += 2;
                }
            }
            if (canonical) {
                FPM_CUDA(fpm::launch_gauge(br.gauge.as<fpm::GaugeTile>(), count, N, M, s));
                br.launches += 1;
            }
        }
    } else if (iters > it0 && br.launch) {
        if (epry || canonical) {
            for (int it = it0; it < iters; ++it) {
                FPM_TRY(engine(it, it + 1));
                if (canonical) {
                    FPM_CUDA(fpm::launch_gauge(br.gauge.as<fpm::GaugeTile>(), count, N, M, s));
                    br.launches += 1;
                }
            }
        } else {
            FPM_TRY(engine(it0, iters));
        }
    }
    if (!br.launch) return Status::ok();
    // Finalise: ifftshift, inverse FFT (FP64) into scratch.
    FPM_CUDA(fpm::launch_state_to_natural(reinterpret_cast<const float2* const*>(br.object_ptrs.ptr),
                                          br.scratch_ptrs.as<double2*>(), count, M, s));
    FPM_TRY(fft2_device(ctx, br.scratch_ptrs.as<double2*>(), count, M, M, true, s));
    br.launches += 3;
    FPM_CUDA(br.record(br.last, s));
    return Status::ok();
}

// Queues one problem's result downloads on stream s: complex64 state is
// widened to complex128 on the device and copied straight into the caller's
// arrays. The status word and objective partials land in the problem's host
// vectors for finish_collect, after the stream is synchronised.
Status queue_collect(fpm_problem* p, const fpm_algorithm_params* a, fpm_result_desc* r, cudaStream_t s) {
    p->host_status = 0;
    FPM_CUDA(cudaMemcpyAsync(&p->host_status, p->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (!r) return Status::ok();
    const int M = p->m, N = p->n, C = fpm::engine_ctas(N);
    const long long ms = M + (M & 1);
    double2* wide = p->scratch64.as<double2>();  // M * M complex128; holds the natural FP64 object first
    if (r->object)
        FPM_CUDA(cudaMemcpyAsync(r->object, wide, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, s));
    if (r->object_spectrum) {
        FPM_CUDA(fpm::launch_widen(p->object.as<float2>(), ms, M, M, wide, s));
        FPM_CUDA(cudaMemcpyAsync(r->object_spectrum, wide, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, s));
    }
    if (r->pupil) {
        FPM_CUDA(fpm::launch_widen(p->pupil_state.as<float2>(), N, N, N, wide, s));
        FPM_CUDA(cudaMemcpyAsync(r->pupil, wide, sizeof(double2) * (size_t)N * N, cudaMemcpyDeviceToHost, s));
    }
    if (r->objectives && a->iterations > 0) {
        p->host_partials.resize((size_t)a->iterations * C);
        FPM_CUDA(cudaMemcpyAsync(p->host_partials.data(), p->partials.ptr, sizeof(double) * p->host_partials.size(),
                                 cudaMemcpyDeviceToHost, s));
    }
    if (r->illumination_corrections && a->algorithm == FPM_ALG_GD && a->recover_illumination)
        FPM_CUDA(cudaMemcpyAsync(r->illumination_corrections, p->ill_correction.ptr, sizeof(double) * 2 * p->frames,
                                 cudaMemcpyDeviceToHost, s));
    if (a->algorithm == FPM_ALG_EPRY && (a->recover_frame_gains || a->recover_background)) {
        if (r->frame_gains)
            FPM_CUDA(cudaMemcpyAsync(r->frame_gains, p->gain_state.ptr, sizeof(double) * p->frames, cudaMemcpyDeviceToHost, s));
        if (r->background) {
            const size_t count = (size_t)N * N * p->frames;
            p->bg_natural.bind(p->ctx->pool, s);
            FPM_TRY(p->bg_natural.ensure(sizeof(double) * count));
            FPM_CUDA(fpm::launch_unpermute_f32_to_f64(N, p->bg_state.as<float>(), p->bg_natural.as<double>(), p->frames, s));
            FPM_CUDA(cudaMemcpyAsync(r->background, p->bg_natural.ptr, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
        }
    }
    return Status::ok();
}

// Weighted mean objective per iteration: the resumed prefix, then the
// per-CTA partials of the iterations this run executed.
void fill_objectives(const fpm_problem* p, const fpm_algorithm_params* a, double* objectives) {
    const int C = fpm::engine_ctas(p->n);
    for (int it = 0; it < a->iterations; ++it) {
        if (it < p->it0) {
            objectives[it] = p->resume_objectives[it];
            continue;
        }
        double sum = 0.0;
        for (int c = 0; c < C; ++c) sum += p->host_partials[(size_t)it * C + c];
        objectives[it] = p->weight_sum > 0.0 ? sum / p->weight_sum : NAN;
    }
}

// Queues the download of one problem's resumable state (after queue_collect
// on the same stream, which it follows in the use of scratch64).
Status queue_capture(fpm_problem* p, const fpm_algorithm_params* a, fpm_state_desc* cap, cudaStream_t s) {
    const int M = p->m, N = p->n, C = fpm::engine_ctas(N);
    const long long ms = M + (M & 1);
    double2* wide = p->scratch64.as<double2>();
    FPM_CUDA(fpm::launch_widen(p->object.as<float2>(), ms, M, M, wide, s));
    FPM_CUDA(cudaMemcpyAsync(cap->object_spectrum, wide, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, s));
    FPM_CUDA(fpm::launch_widen(p->pupil_state.as<float2>(), N, N, N, wide, s));
    FPM_CUDA(cudaMemcpyAsync(cap->pupil, wide, sizeof(double2) * (size_t)N * N, cudaMemcpyDeviceToHost, s));
    if (a->algorithm == FPM_ALG_MPIE) {
        FPM_CUDA(fpm::launch_widen(p->velocity.as<float2>(), ms, M, M, wide, s));
        FPM_CUDA(cudaMemcpyAsync(cap->velocity, wide, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, s));
        FPM_CUDA(fpm::launch_widen(p->anchor.as<float2>(), ms, M, M, wide, s));
        FPM_CUDA(cudaMemcpyAsync(cap->anchor, wide, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, s));
        FPM_CUDA(cudaMemcpyAsync(&p->host_counter, p->counter.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    if (a->iterations > 0) {
        p->host_partials.resize((size_t)a->iterations * C);
        FPM_CUDA(cudaMemcpyAsync(p->host_partials.data(), p->partials.ptr, sizeof(double) * p->host_partials.size(),
                                 cudaMemcpyDeviceToHost, s));
    }
    if (cap->illumination_corrections && a->algorithm == FPM_ALG_GD && a->recover_illumination)
        FPM_CUDA(cudaMemcpyAsync(cap->illumination_corrections, p->ill_correction.ptr, sizeof(double) * 2 * p->frames,
                                 cudaMemcpyDeviceToHost, s));
    return Status::ok();
}

void finish_capture(const fpm_problem* p, const fpm_algorithm_params* a, fpm_state_desc* cap) {
    cap->completed_iterations = a->iterations;
    cap->momentum_counter = a->algorithm == FPM_ALG_MPIE ? p->host_counter : 0;
    if (cap->objectives) fill_objectives(p, a, cap->objectives);
}

Status finish_collect(fpm_problem* p, const fpm_algorithm_params* a, fpm_result_desc* r) {
    const int status = p->host_status;
    if (status & 4) return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "no positive-weight, unmasked measurements are available");
    if (status & 1) return Status::make(FPM_ERR_NUMERICAL, "mPIE momentum produced a non-finite object or velocity");
    if (status & 8) return Status::make(FPM_ERR_NUMERICAL, "object/pupil gauge normalization failed on a non-finite or empty state");
    if (status & 16) return Status::make(FPM_ERR_NUMERICAL, "Poisson truncation statistic is non-finite");
    if (status & 32) return Status::make(FPM_ERR_NUMERICAL, "adaptive alternating projection produced an invalid pass objective");
    if (status & 64) return Status::make(FPM_ERR_NUMERICAL, "pupil update produced a non-finite value");
    if (status & 128) return Status::make(FPM_ERR_NUMERICAL, "regularization produced a non-finite value");
    if (status & 256) return Status::make(FPM_ERR_NUMERICAL, "illumination gradient or curvature is invalid");
    if (status & 512)
        return Status::make(FPM_ERR_TIMEOUT, "a frame-engine stencil load (TMA) did not complete within its bounded wait");
    if (!r) return Status::ok();
    if (r->objectives) fill_objectives(p, a, r->objectives);
    r->completed_iterations = a->iterations;
    return Status::ok();
}

// Device statistics of one batch from the events its buckets recorded
// (synchronises the buckets' streams first).
Status compute_stats(const std::vector<Bucket>& buckets, const std::vector<std::unique_ptr<BucketRun>>& runs,
                     fpm_run_stats& out);

Status record_stats(fpm_context* ctx, const std::vector<Bucket>& buckets,
                    const std::vector<std::unique_ptr<BucketRun>>& runs) {
    for (size_t k = 0; k < buckets.size(); ++k) {
        FPM_CUDA(cudaStreamSynchronize(ctx->streams[k % fpm_context::kStreams]));
        FPM_CUDA(cudaGetLastError());
    }
    return compute_stats(buckets, runs, ctx->stats);
}

// Statistics from the events of finished buckets.
Status compute_stats(const std::vector<Bucket>& buckets, const std::vector<std::unique_ptr<BucketRun>>& runs,
                     fpm_run_stats& out) {
    fpm_run_stats st = {};
    cudaEvent_t first_event = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> engine_events;
    for (size_t k = 0; k < buckets.size(); ++k) {
        if (!first_event) first_event = runs[k]->first;
        for (size_t e = 0; e + 1 < runs[k]->events.size(); e += 2)
            engine_events.emplace_back(runs[k]->events[e], runs[k]->events[e + 1]);
        st.kernel_launches += runs[k]->launches;
        st.engine_bytes += runs[k]->bytes;
    }
    // Spans are measured from the earliest recorded start (the first bucket
    // starts first on the host; later buckets start no earlier).
    for (size_t k = 0; k < buckets.size(); ++k) {
        float last_ms = 0.f;
        FPM_CUDA(cudaEventElapsedTime(&last_ms, first_event, runs[k]->last));
        st.run_ms = std::max(st.run_ms, (double)last_ms);
        if (k < 8) {
            st.bucket_size[k] = buckets[k].n;
            st.bucket_tiles[k] = (int32_t)buckets[k].problems.size();
            st.bucket_end_ms[k] = last_ms;
            st.buckets = (int32_t)k + 1;
        }
    }
    if (!engine_events.empty()) {
        double lo = 1e300, hi = -1e300;
        for (auto& pr : engine_events) {
            float a = 0.f, b = 0.f, d = 0.f;
            FPM_CUDA(cudaEventElapsedTime(&a, first_event, pr.first));
            FPM_CUDA(cudaEventElapsedTime(&b, first_event, pr.second));
            FPM_CUDA(cudaEventElapsedTime(&d, pr.first, pr.second));
            lo = std::min(lo, (double)a);
            hi = std::max(hi, (double)b);
            st.engine_ms_sum += d;
            st.engine_launches += 1;
        }
        st.engine_span_ms = hi - lo;
    }
    out = st;
    return Status::ok();
}

// Checks resumable-state descriptors before any device work.
Status validate_resume(int count, fpm_problem* const* problems, const fpm_algorithm_params* a,
                       const fpm_state_desc* resume, const fpm_state_desc* capture) {
    const bool mpie = a->algorithm == FPM_ALG_MPIE;
    if (resume && a->algorithm == FPM_ALG_ADAPTIVE_AP)
        return Status::make(FPM_ERR_UNSUPPORTED, "adaptive alternating projection does not resume on the GB300 device path");
    if (resume && a->algorithm == FPM_ALG_EPRY && (a->recover_frame_gains || a->recover_background))
        return Status::make(FPM_ERR_UNSUPPORTED,
                            "EPRY runs that recover frame gains or backgrounds do not resume on the GB300 device path");
    for (int i = 0; i < count && resume; ++i) {
        const fpm_state_desc& r = resume[i];
        const fpm_problem* p = problems[i];
        if (r.completed_iterations != resume[0].completed_iterations)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "resumed problems in one batch must share completed_iterations");
        if (r.completed_iterations < 0 || r.completed_iterations > a->iterations)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d: checkpoint has %d completed iterations of %d", i,
                                r.completed_iterations, a->iterations);
        if (!r.object_spectrum || !r.pupil || (r.completed_iterations > 0 && !r.objectives))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d: checkpoint arrays are missing", i);
        if (mpie && (!r.velocity || !r.anchor))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d: mPIE resume needs its velocity and anchor", i);
        if (mpie && (r.momentum_counter < 0 || r.momentum_counter >= a->momentum_interval))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d: momentum counter %d outside [0, %d)", i,
                                r.momentum_counter, a->momentum_interval);
        const size_t m2 = (size_t)p->m * p->m, n2 = (size_t)p->n * p->n;
        auto finite = [](const double* v, size_t n) {
            for (size_t k = 0; k < 2 * n; ++k)
                if (!std::isfinite(v[k])) return false;
            return true;
        };
        const bool illum = a->algorithm == FPM_ALG_GD && a->recover_illumination;
        if (!finite(r.object_spectrum, m2) || !finite(r.pupil, n2) ||
            (mpie && (!finite(r.velocity, m2) || !finite(r.anchor, m2))) ||
            (illum && r.illumination_corrections && !finite(r.illumination_corrections, (size_t)p->frames)))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d: checkpoint holds non-finite values", i);
    }
    for (int i = 0; i < count && capture; ++i) {
        const fpm_state_desc& c = capture[i];
        if (!c.object_spectrum || !c.pupil || (mpie && (!c.velocity || !c.anchor)) || (a->iterations > 0 && !c.objectives))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d: capture arrays are missing", i);
    }
    return Status::ok();
}

// Groups a batch's problems by tile and grid size, largest tiles first so
// the longest launches start earliest; rejects foreign, repeated and busy
// problems.
Status build_buckets(fpm_context* ctx, int count, fpm_problem* const* problems, const fpm_state_desc* resume,
                     std::vector<Bucket>& buckets) {
    if (count < 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "problem count must be non-negative");
    std::vector<const fpm_problem*> seen(problems, problems + count);
    std::sort(seen.begin(), seen.end());
    if (std::adjacent_find(seen.begin(), seen.end()) != seen.end())
        return Status::make(FPM_ERR_INVALID_PARAMETER,
                            "a problem appears twice in one batch; each batched tile needs its own problem (its state is resident)");
    for (int i = 0; i < count; ++i) {
        fpm_problem* p = problems[i];
        if (!p || p->ctx != ctx) return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d does not belong to this context", i);
        if (p->busy) return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d is in use by a submitted job", i);
        if (p->plan) return Status::make(FPM_ERR_INVALID_PARAMETER, "problem %d is held by a captured run plan", i);
        auto it = std::find_if(buckets.begin(), buckets.end(), [&](const Bucket& b) { return b.n == p->n && b.m == p->m; });
        if (it == buckets.end()) {
            buckets.push_back(Bucket{p->n, p->m, {}, {}});
            it = buckets.end() - 1;
        }
        it->problems.push_back(p);
        it->indices.push_back(i);
        if (resume) it->resume.push_back(&resume[i]);
    }
    std::sort(buckets.begin(), buckets.end(), [](const Bucket& x, const Bucket& y) { return x.n > y.n; });
    return Status::ok();
}

Status run_batch(fpm_context* ctx, int count, fpm_problem* const* problems, const fpm_algorithm_params* a,
                 fpm_result_desc* results, const fpm_state_desc* resume = nullptr, fpm_state_desc* capture = nullptr) {
    FPM_TRY(validate_params(a));
    std::vector<Bucket> buckets;
    FPM_TRY(build_buckets(ctx, count, problems, resume, buckets));
    FPM_TRY(validate_resume(count, problems, a, resume, capture));
    std::vector<std::unique_ptr<BucketRun>> runs;
    for (size_t k = 0; k < buckets.size(); ++k) {
        runs.push_back(std::make_unique<BucketRun>());
        FPM_TRY(run_bucket(ctx, buckets[k], a, ctx->streams[k % fpm_context::kStreams], *runs.back()));
    }
    FPM_TRY(record_stats(ctx, buckets, runs));
    for (size_t k = 0; k < buckets.size(); ++k) {
        cudaStream_t s = ctx->streams[k % fpm_context::kStreams];
        for (size_t t = 0; t < buckets[k].problems.size(); ++t) {
            const int idx = buckets[k].indices[t];
            FPM_TRY(queue_collect(buckets[k].problems[t], a, results ? &results[idx] : nullptr, s));
            if (capture) FPM_TRY(queue_capture(buckets[k].problems[t], a, &capture[idx], s));
        }
    }
    for (size_t k = 0; k < buckets.size(); ++k) FPM_CUDA(cudaStreamSynchronize(ctx->streams[k % fpm_context::kStreams]));
    for (size_t k = 0; k < buckets.size(); ++k)
        for (size_t t = 0; t < buckets[k].problems.size(); ++t) {
            const int idx = buckets[k].indices[t];
            FPM_TRY(finish_collect(buckets[k].problems[t], a, results ? &results[idx] : nullptr));
            if (capture) finish_capture(buckets[k].problems[t], a, &capture[idx]);
        }
    return Status::ok();
}

// Host-input batch: problems are created, run and downloaded in chunks so
// that the host validation and upload of chunk k + 1 overlap the run of
// chunk k, and the downloads of finished chunks overlap the runs still in
// flight. Chunks follow run_batch's order (largest tiles first) and hold at
// most kChunkBytes of float64 measurements.
Status run_batch_host(fpm_context* ctx, int count, const fpm_model_desc* mds, const fpm_measurement_desc* mss,
                      const fpm_algorithm_params* a, fpm_result_desc* results,
                      std::vector<std::unique_ptr<fpm_problem>>& made) {
    constexpr size_t kChunkBytes = size_t(1) << 31;
    using clock = std::chrono::steady_clock;
    const auto t_call = clock::now();
    auto since = [](clock::time_point t0) {
        return std::chrono::duration<double, std::milli>(clock::now() - t0).count();
    };
    double scan_ms = 0.0, upload_ms = 0.0, first_launch_ms = 0.0;
    FPM_TRY(validate_params(a));
    if (count < 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "problem count must be non-negative");
    made.clear();
    made.resize(count);
    std::vector<size_t> bytes(count);
    for (int i = 0; i < count; ++i) {
        Status st = validate_model(&mds[i]);
        if (!st) st = check_measurement_header(&mds[i], &mss[i]);
        if (st) return Status::make(st.code, "problem %d: %s", i, st.message.c_str());
        bytes[i] = (size_t)mds[i].image_height * mds[i].image_width * mss[i].frames * sizeof(double);
    }
    // Buckets by (n, m), largest tiles first, then chunks.
    std::vector<std::pair<std::pair<int, int>, std::vector<int>>> groups;
    for (int i = 0; i < count; ++i) {
        const std::pair<int, int> key(mds[i].image_height, mds[i].recon_height);
        auto it = std::find_if(groups.begin(), groups.end(), [&](const auto& g) { return g.first == key; });
        if (it == groups.end()) {
            groups.push_back({key, {}});
            it = groups.end() - 1;
        }
        it->second.push_back(i);
    }
    std::stable_sort(groups.begin(), groups.end(), [](const auto& x, const auto& y) { return x.first.first > y.first.first; });
    std::vector<Bucket> chunks;
    for (const auto& g : groups) {
        // Sizes whose engine picks its shape by the launch's tile count
        // keep enough tiles per chunk for the single-CTA engine. The first
        // chunk stays an ordinary one when the rest still fills such chunks:
        // it runs on the cluster engine while the large chunks upload, so
        // the device starts after one chunk's upload rather than a large one.
        size_t min_tiles = 1, first_tiles = 0;
        {
            bool single = false;
            int resident = 0;
            const bool amplitude = mds[g.second[0]].background == nullptr;
            const bool recovery = a->algorithm == FPM_ALG_EPRY && (a->recover_frame_gains || a->recover_background);
            FPM_TRY(single_cta_engine(ctx, g.first.first, engine_family(a),
                                      amplitude && !a->compensated_accumulation && !recovery, (int)g.second.size(),
                                      &single, &resident));
            if (single) {
                const size_t threshold = std::max(1, (2 * resident + 2) / 3);
                size_t head = 0, head_bytes = 0;
                for (int i : g.second) {
                    if (head > 0 && head_bytes + bytes[i] > kChunkBytes) break;
                    head_bytes += bytes[i];
                    ++head;
                }
                const size_t rest = g.second.size() - head;
                if (head < g.second.size() && rest >= threshold) first_tiles = head;
                const size_t pool = first_tiles ? rest : g.second.size();
                const size_t parts = std::max<size_t>(1, pool / threshold);
                min_tiles = (pool + parts - 1) / parts;
            }
        }
        size_t acc = 0, tiles = 0, placed = 0;
        for (int i : g.second) {
            const size_t need = first_tiles && placed < first_tiles ? first_tiles : min_tiles;
            const bool head_done = first_tiles && placed == first_tiles;
            if (chunks.empty() || chunks.back().n != g.first.first || chunks.back().m != g.first.second ||
                head_done || (acc + bytes[i] > kChunkBytes && tiles >= need)) {
                chunks.push_back(Bucket{g.first.first, g.first.second, {}, {}});
                acc = 0;
                tiles = 0;
            }
            ++placed;
            chunks.back().indices.push_back(i);
            acc += bytes[i];
            ++tiles;
        }
    }
    std::vector<std::unique_ptr<BucketRun>> runs;
    for (size_t k = 0; k < chunks.size(); ++k) {
        Bucket& ch = chunks[k];
        std::vector<long long> first(ch.indices.size() + 1, 0);
        for (size_t t = 0; t < ch.indices.size(); ++t) first[t + 1] = first[t] + mss[ch.indices[t]].frames;
        std::vector<FrameScan> scans(first.back());
        std::vector<int> owner(first.back());
        for (size_t t = 0; t < ch.indices.size(); ++t)
            for (long long q = first[t]; q < first[t + 1]; ++q) owner[q] = (int)t;
        const auto t_scan = clock::now();
        HostPool::get().run(first.back(), [&](long long q) {
            const int i = ch.indices[owner[q]];
            scan_frame(&mds[i], &mss[i], (int)(q - first[owner[q]]), scans[q]);
        });
        scan_ms += since(t_scan);
        for (size_t t = 0; t < ch.indices.size(); ++t) {
            const int i = ch.indices[t];
            Status st = check_scans(&mss[i], scans.data() + first[t]);
            if (!st) st = prepare_problem(ctx, &mds[i], &mss[i], scans.data() + first[t], made[i]);
            if (st) return Status::make(st.code, "problem %d: %s", i, st.message.c_str());
            const auto t_up = clock::now();
            FPM_TRY(upload_problem(ctx, made[i].get(), &mds[i], &mss[i], ctx->upload));
            upload_ms += since(t_up);
            ch.problems.push_back(made[i].get());
        }
        cudaEvent_t ready;
        FPM_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
        FPM_CUDA(cudaEventRecord(ready, ctx->upload));
        cudaStream_t s = ctx->streams[k % fpm_context::kStreams];
        const cudaError_t wait = cudaStreamWaitEvent(s, ready, 0);
        cudaEventDestroy(ready);
        FPM_CUDA(wait);
        runs.push_back(std::make_unique<BucketRun>());
        FPM_TRY(run_bucket(ctx, ch, a, s, *runs.back()));
        if (k == 0) first_launch_ms = since(t_call);
    }
    // Downloads on their own stream, chunk by chunk in the order the chunks
    // finish (polled on each chunk's last event), so a chunk's results reach
    // the host as soon as its own work is done; the time each arrives is its
    // tiles' latency from the call's start.
    std::vector<double> done_ms(chunks.size(), -1.0);
    for (size_t left = chunks.size(); left > 0;) {
        bool progressed = false;
        for (size_t k = chunks.size(); k-- > 0;) {
            if (done_ms[k] >= 0.0) continue;
            const cudaError_t q = cudaEventQuery(runs[k]->last);
            if (q == cudaErrorNotReady) continue;
            FPM_CUDA(q);
            FPM_CUDA(cudaStreamWaitEvent(ctx->download, runs[k]->last, 0));
            for (size_t t = 0; t < chunks[k].problems.size(); ++t) {
                const int idx = chunks[k].indices[t];
                FPM_TRY(queue_collect(chunks[k].problems[t], a, results ? &results[idx] : nullptr, ctx->download));
            }
            FPM_CUDA(cudaStreamSynchronize(ctx->download));
            done_ms[k] = since(t_call);
            --left;
            progressed = true;
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    for (size_t k = 0; k < chunks.size(); ++k) FPM_CUDA(cudaStreamSynchronize(ctx->streams[k % fpm_context::kStreams]));
    FPM_TRY(record_stats(ctx, chunks, runs));
    ctx->stats.host_first_launch_ms = first_launch_ms;
    ctx->stats.host_scan_ms = scan_ms;
    ctx->stats.host_upload_ms = upload_ms;
    ctx->stats.host_call_ms = since(t_call);
    ctx->stats.host_chunks = (int32_t)std::min<size_t>(chunks.size(), 16);
    for (size_t k = 0; k < chunks.size() && k < 16; ++k) {
        ctx->stats.host_done_ms[k] = done_ms[k];
        ctx->stats.host_done_tiles[k] = (int32_t)chunks[k].problems.size();
    }
    for (size_t k = 0; k < chunks.size(); ++k)
        for (size_t t = 0; t < chunks[k].problems.size(); ++t) {
            const int idx = chunks[k].indices[t];
            FPM_TRY(finish_collect(chunks[k].problems[t], a, results ? &results[idx] : nullptr));
        }
    return Status::ok();
}

// ------------------------------------------------------------ spectral AP

// SpectralImagePlaneModel::validate (src/model/spectral.rs:302-398),
// SpectralReconstructionProblem::validate (src/reconstruction/spectral.rs:
// 55-92) and SpectralAlternatingProjection::validate
// (src/algorithms/spectral.rs:149-173), before any device work.
Status validate_spectral(const fpm_spectral_model_desc* sm, const fpm_measurement_desc* ms,
                         const fpm_spectral_params* a) {
    if (!sm || !ms || !a) return Status::make(FPM_ERR_INVALID_PARAMETER, "spectral model, measurements and parameters are required");
    if (!std::isfinite(a->object_step) || a->object_step <= 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "object_step must be finite and positive");
    if (!std::isfinite(a->epsilon) || a->epsilon <= 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "epsilon must be finite and positive");
    if (a->iterations <= 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "iterations must be positive");
    if (a->batch_size <= 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "batch_size must be positive");
    if (a->loss_type < 0 || a->loss_type > 3) return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown loss type %d", a->loss_type);
    if (sm->channels <= 0 || !sm->channel_models)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "at least one spectral channel is required");
    if (sm->object_coupling != FPM_COUPLING_INDEPENDENT && sm->object_coupling != FPM_COUPLING_SHARED_COMPLEX)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown object coupling %d", sm->object_coupling);
    const fpm_model_desc& c0 = sm->channel_models[0];
    for (int c = 0; c < sm->channels; ++c) {
        const fpm_model_desc& md = sm->channel_models[c];
        FPM_TRY(validate_model(&md));
        if (md.image_height != c0.image_height || md.image_width != c0.image_width ||
            md.recon_height != c0.recon_height || md.recon_width != c0.recon_width)
            return Status::make(FPM_ERR_INVALID_PARAMETER,
                                "all channel kernels must share detector shape, reconstruction grid, and object-plane pixel pitch");
        if (md.background)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "background belongs to physical detector rows, not channel kernels");
    }
    const int N = c0.image_height;
    if (c0.image_width != N || !fpm::engine_supported(N) || c0.recon_width != c0.recon_height)
        return Status::make(FPM_ERR_UNSUPPORTED,
                            "the GB300 device path reconstructs square tiles of 32, 64, 128 or 256 pixels on a square grid");
    const int E = sm->exposures;
    if (E <= 0 || !sm->contribution_offsets || !sm->exposure_gain || !sm->exposure_background)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "at least one detector frame is required");
    if (sm->contribution_offsets[0] != 0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "contribution offsets must start at zero");
    std::vector<std::vector<char>> covered(sm->channels), positive(sm->channels);
    for (int c = 0; c < sm->channels; ++c) {
        covered[c].assign(sm->channel_models[c].sources, 0);
        positive[c].assign(sm->channel_models[c].sources, 0);
    }
    for (int e = 0; e < E; ++e) {
        const int first = sm->contribution_offsets[e], last = sm->contribution_offsets[e + 1];
        if (last <= first) return Status::make(FPM_ERR_INVALID_PARAMETER, "each detector frame must have a positive contribution");
        if (!std::isfinite(sm->exposure_gain[e]) || sm->exposure_gain[e] <= 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "spectral frame gain must be finite and positive");
        if (!std::isfinite(sm->exposure_background[e]) || sm->exposure_background[e] < 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "spectral frame background must be finite and non-negative");
        double mode_weight_sum = 0.0;
        for (int k = first; k < last; ++k) {
            const int c = sm->contribution_channel[k], l = sm->contribution_local_frame[k];
            if (c < 0 || c >= sm->channels || l < 0 || l >= sm->channel_models[c].sources)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "channel/local_frame reference is out of range");
            for (int j = first; j < k; ++j)
                if (sm->contribution_channel[j] == c && sm->contribution_local_frame[j] == l)
                    return Status::make(FPM_ERR_INVALID_PARAMETER, "duplicate (channel, local_frame) contribution in frame %d", e);
            const double w = sm->contribution_weight[k];
            if (!std::isfinite(w) || w <= 0.0)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "spectral weights must be finite and positive");
            covered[c][l] = 1;
            const double fg = sm->channel_models[c].frame_gains ? sm->channel_models[c].frame_gains[l] : 1.0;
            mode_weight_sum += w * fg;
        }
        if (!std::isfinite(mode_weight_sum) || mode_weight_sum <= 0.0 ||
            !std::isfinite(sm->exposure_gain[e] * mode_weight_sum) || sm->exposure_gain[e] * mode_weight_sum <= 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "effective source-mode weight sum must be finite and positive");
    }
    for (auto& v : covered)
        for (char x : v)
            if (!x) return Status::make(FPM_ERR_INVALID_PARAMETER, "every channel and local frame must participate in the detector plan");
    if (ms->frames != E || !ms->measurements)
        return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "spectral detector frame count and shape must match the compiled model");
    const size_t n2 = (size_t)N * N;
    for (size_t i = 0; i < n2 * E; ++i)
        if (!std::isfinite(ms->measurements[i]))
            return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "measurements contain non-finite values");
    for (int e = 0; e < E; ++e) {
        const double w = ms->frame_weights ? ms->frame_weights[e] : 1.0;
        if (!std::isfinite(w) || w < 0.0)
            return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "frame weights must be finite and non-negative");
        if (w == 0.0) continue;
        if (ms->masks) {
            bool any = false;
            for (size_t i = 0; i < n2 && !any; ++i) any = ms->masks[(size_t)e * n2 + i] != 0;
            if (!any) return Status::make(FPM_ERR_INVALID_MEASUREMENTS, "positive-weight frame %d has no unmasked pixels", e);
        }
        for (int k = sm->contribution_offsets[e]; k < sm->contribution_offsets[e + 1]; ++k)
            positive[sm->contribution_channel[k]][sm->contribution_local_frame[k]] = 1;
    }
    for (auto& v : positive)
        for (char x : v)
            if (!x)
                return Status::make(FPM_ERR_INVALID_MEASUREMENTS,
                                    "every spectral channel and local frame must participate in a positive-weight detector frame");
    return Status::ok();
}

double spectral_frame_gain(const fpm_spectral_model_desc* sm, int c, int l) {
    return sm->channel_models[c].frame_gains ? sm->channel_models[c].frame_gains[l] : 1.0;
}

// SpectralReconstructionState::initialize (src/reconstruction/spectral.rs:
// 123-199) on the host in FP64: per stored object, the weighted mask-aware
// mean of sqrt(max((I - background) / gain, 0)) over the exposures that use
// it, nearest-upsampled to the common grid (natural order, complex128).
Status spectral_initial_objects(const fpm_spectral_model_desc* sm, const fpm_measurement_desc* ms, int objects,
                                std::vector<double>& out) {
    const fpm_model_desc& c0 = sm->channel_models[0];
    const int h = c0.image_height, w = c0.image_width, mh = c0.recon_height, mw = c0.recon_width;
    const size_t n = (size_t)h * w, nm = (size_t)mh * mw;
    out.assign(2 * nm * objects, 0.0);
    std::vector<double> amplitude(n), weights(n);
    for (int o = 0; o < objects; ++o) {
        std::fill(amplitude.begin(), amplitude.end(), 0.0);
        std::fill(weights.begin(), weights.end(), 0.0);
        double total_amplitude = 0.0, total_weight = 0.0;
        for (int e = 0; e < sm->exposures; ++e) {
            const int first = sm->contribution_offsets[e], last = sm->contribution_offsets[e + 1];
            bool uses = false;
            for (int k = first; k < last; ++k)
                uses |= (sm->object_coupling == FPM_COUPLING_SHARED_COMPLEX ? 0 : sm->contribution_channel[k]) == o;
            if (!uses) continue;
            const double fw = ms->frame_weights ? ms->frame_weights[e] : 1.0;
            if (fw == 0.0) continue;
            double gain = 0.0;
            for (int k = first; k < last; ++k)
                gain += sm->contribution_weight[k] *
                        spectral_frame_gain(sm, sm->contribution_channel[k], sm->contribution_local_frame[k]);
            gain *= sm->exposure_gain[e];
            if (!std::isfinite(gain) || gain <= 0.0)
                return Status::make(FPM_ERR_NUMERICAL, "spectral initialization gain must be finite and positive");
            const double* m = ms->measurements + (size_t)e * n;
            const uint8_t* mk = ms->masks ? ms->masks + (size_t)e * n : nullptr;
            const double bg = sm->exposure_background[e];
            for (size_t i = 0; i < n; ++i) {
                if (mk && mk[i] == 0) continue;
                const double value = std::sqrt(std::max((m[i] - bg) / gain, 0.0));
                amplitude[i] += fw * value;
                weights[i] += fw;
                total_amplitude += fw * value;
                total_weight += fw;
            }
        }
        const double fallback = total_amplitude / total_weight;
        for (size_t i = 0; i < n; ++i) amplitude[i] = weights[i] > 0.0 ? amplitude[i] / weights[i] : fallback;
        double* obj = out.data() + 2 * nm * o;
        for (long long r = 0; r < mh; ++r)
            for (long long c = 0; c < mw; ++c) obj[2 * (r * mw + c)] = amplitude[(r * h / mh) * w + c * w / mw];
    }
    return Status::ok();
}

// One spectral reconstruction on the device: host constants, resident
// buffers and the result downloads.
struct SpectralJob {
    const fpm_spectral_model_desc* sm = nullptr;
    const fpm_measurement_desc* ms = nullptr;
    int N = 0, M = 0, E = 0, CH = 0, objects = 0, completed = 0, max_modes = 1;
    long long ostride = 0;
    double weight_total = 0.0, bytes_per_pass = 0.0;
    std::vector<fpm::FrameParam> params;
    std::vector<fpm::SpectralStep> steps;
    std::vector<float2> pupils;
    std::vector<double> natural;
    const double* start_objects = nullptr;
    const double* resume_spectra = nullptr;
    std::vector<float2*> optr;
    std::vector<double2*> wptr;
    std::vector<double> host_partials;
    int host_status = 0;
    DeviceBuffer meas, masks, d_pupils, d_params, d_steps, object, wide, fields, prediction, partials, status,
        object_ptrs, wide_ptrs;
};

// Host part of SpectralRunner::run with SpectralAlternatingProjection
// (src/reconstruction/spectral.rs:494-642, src/algorithms/spectral.rs:
// 182-271): validation, crops, the virtual steps of one pass in schedule
// order (each exposure's evaluation steps, then its update steps) and the
// starting objects.
Status spectral_prepare(SpectralJob& j, const fpm_spectral_model_desc* sm, const fpm_measurement_desc* ms,
                        const fpm_spectral_params* a, const int32_t* order, const double* initial_objects,
                        const double* resume_spectra, int completed) {
    FPM_TRY(validate_spectral(sm, ms, a));
    if (completed < 0 || completed > a->iterations)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "total target cannot precede checkpoint iterations");
    if (initial_objects && resume_spectra)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "cannot combine initial objects with a checkpoint");
    if (completed > 0 && !resume_spectra)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "completed iterations need the checkpoint's spectra");
    const fpm_model_desc& c0 = sm->channel_models[0];
    j.sm = sm;
    j.ms = ms;
    j.N = c0.image_height;
    j.M = c0.recon_height;
    j.E = sm->exposures;
    j.CH = sm->channels;
    j.objects = sm->object_coupling == FPM_COUPLING_SHARED_COMPLEX ? 1 : j.CH;
    j.ostride = j.M + (j.M & 1);
    j.completed = completed;
    const int N = j.N, M = j.M, E = j.E, CH = j.CH;
    const size_t n2 = (size_t)N * N, nm = (size_t)M * M;
    std::vector<int> schedule(E);
    for (int e = 0; e < E; ++e) schedule[e] = e;
    if (order) {
        std::vector<char> seen(E, 0);
        for (int e = 0; e < E; ++e) {
            if (order[e] < 0 || order[e] >= E || seen[order[e]])
                return Status::make(FPM_ERR_INVALID_PARAMETER, "explicit order must be a permutation of all detector frames");
            seen[order[e]] = 1;
            schedule[e] = order[e];
        }
    }
    for (const double* arr : {initial_objects, resume_spectra})
        if (arr)
            for (size_t i = 0; i < 2 * nm * j.objects; ++i)
                if (!std::isfinite(arr[i])) return Status::make(FPM_ERR_INVALID_PARAMETER, "complex values must be finite");

    // Crops of every channel source; FrameParam k = source_offset[c] + l.
    std::vector<int> source_offset(CH + 1, 0);
    for (int c = 0; c < CH; ++c) source_offset[c + 1] = source_offset[c] + sm->channel_models[c].sources;
    j.params.assign(source_offset[CH], fpm::FrameParam{});
    std::vector<double> stencil(source_offset[CH]);
    for (int c = 0; c < CH; ++c) {
        const fpm_model_desc& md = sm->channel_models[c];
        for (int l = 0; l < md.sources; ++l) {
            fpm::FrameParam& fp = j.params[source_offset[c] + l];
            FPM_TRY(crop_frame_param(md.crop_start_row[l], md.crop_start_col[l], md.offset_row ? md.offset_row[l] : 0.0,
                                     md.offset_col ? md.offset_col[l] : 0.0, N, M, fp));
            fp.weight = 1.f;
            fp.gain = 1.f;
            stencil[source_offset[c] + l] = (double)(N + fp.has_upper_row) * (double)(N + fp.has_upper_col);
        }
    }
    j.steps.clear();
    for (int idx = 0; idx < E; ++idx) {
        const int e = schedule[idx];
        const double fw = ms->frame_weights ? ms->frame_weights[e] : 1.0;
        if (fw == 0.0) continue;
        const int first = sm->contribution_offsets[e], count = sm->contribution_offsets[e + 1] - first;
        j.max_modes = std::max(j.max_modes, count);
        const bool separate = count == 1;
        double gain = sm->exposure_gain[e];
        if (separate)
            gain *= sm->contribution_weight[first] *
                    spectral_frame_gain(sm, sm->contribution_channel[first], sm->contribution_local_frame[first]);
        std::vector<double> wk(count);
        double wsum = 0.0;
        for (int k = 0; k < count; ++k) {
            const int c = sm->contribution_channel[first + k], l = sm->contribution_local_frame[first + k];
            wk[k] = separate ? 1.0 : sm->contribution_weight[first + k] * spectral_frame_gain(sm, c, l);
            wsum += wk[k];
        }
        long long valid = (long long)n2;
        if (ms->masks) {
            valid = 0;
            for (size_t i = 0; i < n2; ++i) valid += ms->masks[(size_t)e * n2 + i] != 0;
        }
        j.weight_total += fw;
        // Evaluations 0..K-1 (the last one also updates its mode), then the
        // updates K-2..0.
        std::vector<std::pair<int, int>> order;  // (mode position, step kind)
        for (int k = 0; k < count; ++k) order.emplace_back(k, k == count - 1 ? 2 : 0);
        for (int k = count - 2; k >= 0; --k) order.emplace_back(k, 1);
        for (const auto& [k, kind] : order) {
            const int c = sm->contribution_channel[first + k], l = sm->contribution_local_frame[first + k];
            fpm::SpectralStep st{};
            const int mode = source_offset[c] + l;
            st.frame = j.params[mode];
            st.exposure = e;
            st.object = sm->object_coupling == FPM_COUPLING_SHARED_COMPLEX ? 0 : c;
            st.channel = c;
            st.update = kind;
            st.slot = k;
            st.mode_weight = (float)wk[k];
            st.update_scale = (float)(fw * (wk[k] / wsum));
            st.gain = (float)gain;
            st.background = (float)sm->exposure_background[e];
            st.inv_weight_sum = (float)(1.0 / wsum);
            st.first_update = kind == 2 ? 1 : 0;
            st.loss_scale = fw / (double)valid;
            j.steps.push_back(st);
            // Algorithmic HBM bytes: stencil read (evaluation), object
            // read-modify-write (update), measurement (+ mask) once.
            j.bytes_per_pass += (kind != 1 ? 8.0 : 0.0) * stencil[mode] + (kind != 0 ? 16.0 : 0.0) * stencil[mode];
        }
        j.bytes_per_pass += 4.0 * (double)n2 + (ms->masks ? (double)n2 : 0.0);
    }
    if (!(j.weight_total > 0.0)) return Status::make(FPM_ERR_NUMERICAL, "spectral iteration has no positive frame weight");
    j.resume_spectra = resume_spectra;
    if (!resume_spectra && !initial_objects) FPM_TRY(spectral_initial_objects(sm, ms, j.objects, j.natural));
    j.start_objects = initial_objects ? initial_objects : j.natural.data();
    j.pupils.resize(n2 * CH);
    for (int c = 0; c < CH; ++c)
        for (size_t i = 0; i < n2; ++i)
            j.pupils[c * n2 + i] = make_float2((float)sm->channel_models[c].pupil[2 * i],
                                               (float)sm->channel_models[c].pupil[2 * i + 1]);
    return Status::ok();
}

// Device part: resident buffers from the context's pool, measurements in the
// engine's FP32 layout (raw form: per-exposure gain and background), and the
// starting state, queued on stream s.
Status spectral_upload(fpm_context* ctx, SpectralJob& j, const fpm_spectral_params* a, cudaStream_t s, int& launches) {
    const int N = j.N, M = j.M, E = j.E, C = fpm::engine_ctas(N);
    const size_t n2 = (size_t)N * N, nm = (size_t)M * M;
    for (DeviceBuffer* b : {&j.meas, &j.masks, &j.d_pupils, &j.d_params, &j.d_steps, &j.object, &j.wide, &j.fields,
                            &j.prediction, &j.partials, &j.status, &j.object_ptrs, &j.wide_ptrs})
        b->bind(ctx->pool, s);
    const size_t total = n2 * E;
    // Staging from the pool, freed (stream-ordered) once permuted: jobs in
    // flight never share it.
    DeviceBuffer staging, mask_staging;
    staging.bind(ctx->pool, s);
    mask_staging.bind(ctx->pool, s);
    FPM_TRY(staging.ensure(total * sizeof(double)));
    FPM_TRY(j.meas.ensure(total * sizeof(float)));
    FPM_CUDA(cudaMemcpyAsync(staging.ptr, j.ms->measurements, total * sizeof(double), cudaMemcpyHostToDevice, s));
    FPM_CUDA(fpm::launch_permute_f64_to_f32(N, staging.as<double>(), j.meas.as<float>(), E, s));
    ++launches;
    if (j.ms->masks) {
        FPM_TRY(j.masks.ensure(total));
        FPM_TRY(mask_staging.ensure(total));
        FPM_CUDA(cudaMemcpyAsync(mask_staging.ptr, j.ms->masks, total, cudaMemcpyHostToDevice, s));
        FPM_CUDA(fpm::launch_permute_u8(N, mask_staging.as<uint8_t>(), j.masks.as<uint8_t>(), E, s));
        ++launches;
    }
    FPM_TRY(upload_array(ctx, j.d_pupils, j.pupils, s));
    FPM_TRY(upload_array(ctx, j.d_steps, j.steps, s));
    FPM_TRY(j.object.ensure(sizeof(float2) * (size_t)M * j.ostride * j.objects));
    FPM_TRY(j.wide.ensure(sizeof(double2) * nm * j.objects));
    FPM_TRY(j.fields.ensure(sizeof(float2) * n2 * j.max_modes));
    FPM_TRY(j.prediction.ensure(sizeof(float) * n2));
    FPM_TRY(j.partials.ensure(sizeof(double) * (size_t)a->iterations * C));
    FPM_TRY(j.status.ensure(sizeof(int)));
    FPM_CUDA(cudaMemsetAsync(j.status.ptr, 0, sizeof(int), s));
    FPM_CUDA(cudaMemsetAsync(j.partials.ptr, 0, sizeof(double) * (size_t)a->iterations * C, s));
    j.optr.resize(j.objects);
    j.wptr.resize(j.objects);
    for (int o = 0; o < j.objects; ++o) {
        j.optr[o] = j.object.as<float2>() + (size_t)o * M * j.ostride;
        j.wptr[o] = j.wide.as<double2>() + (size_t)o * nm;
    }
    FPM_TRY(upload_array(ctx, j.object_ptrs, j.optr, s));
    FPM_TRY(upload_array(ctx, j.wide_ptrs, j.wptr, s));
    if (j.resume_spectra) {
        // Checkpoint spectra are the widened complex64 state: narrowing restores it exactly.
        FPM_CUDA(cudaMemcpyAsync(j.wide.ptr, j.resume_spectra, sizeof(double2) * nm * j.objects, cudaMemcpyHostToDevice, s));
        for (int o = 0; o < j.objects; ++o) FPM_CUDA(fpm::launch_narrow(j.wptr[o], M, M, j.optr[o], j.ostride, s));
        launches += j.objects;
    } else {
        // Forward FFT (FP64) and fftshift of the natural-order objects.
        FPM_CUDA(cudaMemcpyAsync(j.wide.ptr, j.start_objects, sizeof(double2) * nm * j.objects, cudaMemcpyHostToDevice, s));
        FPM_TRY(fft2_device(ctx, j.wide_ptrs.as<double2*>(), j.objects, M, M, false, s));
        FPM_CUDA(fpm::launch_shift_to_state(j.wide_ptrs.as<double2*>(), j.object_ptrs.as<float2*>(), nullptr, nullptr,
                                            j.objects, M, s));
        launches += 3;
    }
    return Status::ok();
}

fpm::TileDesc spectral_tile(const SpectralJob& j) {
    fpm::TileDesc T{};
    T.object = j.object.as<float2>();
    T.pupil = j.d_pupils.as<float2>();
    T.meas = j.meas.as<float>();
    T.masks = j.ms->masks ? j.masks.as<uint8_t>() : nullptr;
    T.params = nullptr;  // each step carries its crop
    T.partials = j.partials.as<double>();
    T.status = j.status.as<int>();
    T.M = j.M;
    T.frame_count = j.E;
    T.max_pupil_power = 1.0;
    T.weight_sum = j.weight_total;
    T.row_lo = 0;
    T.row_hi = j.N - 1;
    T.steps = j.d_steps.as<fpm::SpectralStep>();
    T.step_count = (int)j.steps.size();
    T.mode_fields = j.fields.as<float2>();
    T.prediction = j.prediction.as<float>();
    return T;
}

fpm::EngineParams spectral_engine_params(const fpm_spectral_params* a, int completed) {
    fpm::EngineParams ep{};
    ep.alg = fpm::kAlgSpectral;
    ep.eps = a->epsilon;
    ep.object_step = a->object_step;
    ep.loss = a->loss_type;
    ep.gd_batch = 1;
    ep.it_begin = completed;
    ep.it_end = a->iterations;
    return ep;
}

// Final objects (ifftshift, FP64 inverse FFT) and the result downloads on s.
Status spectral_queue_collect(fpm_context* ctx, SpectralJob& j, const fpm_spectral_params* a, cudaStream_t s,
                              double* objects_out, double* spectra_out, int& launches) {
    const int M = j.M, C = fpm::engine_ctas(j.N);
    const size_t nm = (size_t)M * M;
    FPM_CUDA(fpm::launch_state_to_natural(reinterpret_cast<const float2* const*>(j.object_ptrs.ptr),
                                          j.wide_ptrs.as<double2*>(), j.objects, M, s));
    FPM_TRY(fft2_device(ctx, j.wide_ptrs.as<double2*>(), j.objects, M, M, true, s));
    launches += 3;
    if (objects_out)
        FPM_CUDA(cudaMemcpyAsync(objects_out, j.wide.ptr, sizeof(double2) * nm * j.objects, cudaMemcpyDeviceToHost, s));
    if (spectra_out) {
        // The natural objects leave j.wide first (stream order), then the spectra reuse it.
        for (int o = 0; o < j.objects; ++o) FPM_CUDA(fpm::launch_widen(j.optr[o], j.ostride, M, M, j.wptr[o], s));
        launches += j.objects;
        FPM_CUDA(cudaMemcpyAsync(spectra_out, j.wide.ptr, sizeof(double2) * nm * j.objects, cudaMemcpyDeviceToHost, s));
    }
    j.host_partials.resize((size_t)a->iterations * C);
    FPM_CUDA(cudaMemcpyAsync(j.host_partials.data(), j.partials.ptr, sizeof(double) * j.host_partials.size(),
                             cudaMemcpyDeviceToHost, s));
    FPM_CUDA(cudaMemcpyAsync(&j.host_status, j.status.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    return Status::ok();
}

// Pass objectives from the per-CTA partials, after the stream is synchronised.
Status spectral_objectives(const SpectralJob& j, const fpm_spectral_params* a, double* objectives_out) {
    const int C = fpm::engine_ctas(j.N);
    for (int it = j.completed; it < a->iterations; ++it) {
        double sum = 0.0;
        for (int r = 0; r < C; ++r) sum += j.host_partials[(size_t)it * C + r];
        const double objective = sum / j.weight_total;
        if (!std::isfinite(objective)) return Status::make(FPM_ERR_NUMERICAL, "spectral iteration objective is non-finite");
        if (objectives_out) objectives_out[it - j.completed] = objective;
    }
    return Status::ok();
}

// Device timeline of a spectral batch: its events and launch buffers,
// kept until the work has finished.
struct SpectralBatch {
    std::vector<cudaEvent_t> ev;
    cudaEvent_t start = nullptr, uploaded = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> engine_events;
    std::vector<cudaEvent_t> ends;
    std::vector<std::unique_ptr<DeviceBuffer>> tile_bufs;
    std::vector<int> groups;  // job indices in launch order, per tile size
    fpm_run_stats st{};
    int launches = 0;
    ~SpectralBatch() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    Status event(cudaEvent_t& e) {
        FPM_CUDA(cudaEventCreate(&e));
        ev.push_back(e);
        return Status::ok();
    }
};

// Queues jobs on the device: uploads on streams[0], then one engine launch
// per tile size over all its jobs (one cluster each), the largest (longest)
// tiles first so that they take SMs before the short ones, sizes on
// separate streams. With `collect` the finalisation and result downloads
// follow on the same streams.
Status spectral_queue(fpm_context* ctx, std::vector<SpectralJob>& jobs, const fpm_spectral_params* a,
                      const std::vector<fpm_spectral_result_desc>& results, const std::vector<cudaStream_t>& streams,
                      bool collect, SpectralBatch& b) {
    FPM_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s0 = streams[0];
    FPM_TRY(b.event(b.start));
    FPM_TRY(b.event(b.uploaded));
    FPM_CUDA(cudaEventRecord(b.start, s0));
    for (SpectralJob& j : jobs) FPM_TRY(spectral_upload(ctx, j, a, s0, b.launches));
    FPM_CUDA(cudaEventRecord(b.uploaded, s0));
    std::map<int, std::vector<int>, std::greater<int>> by_size;
    for (size_t i = 0; i < jobs.size(); ++i) by_size[jobs[i].N].push_back((int)i);
    size_t k = 0;
    for (auto& [N, idx] : by_size) {
        cudaStream_t s = streams[k % streams.size()];
        FPM_CUDA(cudaStreamWaitEvent(s, b.uploaded, 0));
        std::vector<fpm::TileDesc> tiles;
        double bytes = 0.0;
        int completed = jobs[idx[0]].completed;
        for (int i : idx) {
            tiles.push_back(spectral_tile(jobs[i]));
            bytes += jobs[i].bytes_per_pass * (a->iterations - jobs[i].completed);
            if (jobs[i].completed != completed)
                return Status::make(FPM_ERR_INVALID_PARAMETER, "every resumed problem must have the same completed iterations");
        }
        b.tile_bufs.push_back(std::make_unique<DeviceBuffer>());
        b.tile_bufs.back()->bind(ctx->pool, s);
        FPM_TRY(upload_array(ctx, *b.tile_bufs.back(), tiles, s));
        fpm::EngineParams ep = spectral_engine_params(a, completed);
        ep.tiles = b.tile_bufs.back()->as<fpm::TileDesc>();
        ep.tile_count = (int)tiles.size();
        cudaEvent_t e0, e1, done;
        FPM_TRY(b.event(e0));
        FPM_TRY(b.event(e1));
        FPM_TRY(b.event(done));
        FPM_CUDA(cudaEventRecord(e0, s));
        if (a->iterations > completed) {
            FPM_CUDA(fpm::launch_engine(N, ep, engine_clusters(ctx, N, (int)tiles.size()), s));
            ++b.launches;
            b.st.engine_launches += 1;
        }
        FPM_CUDA(cudaEventRecord(e1, s));
        b.engine_events.emplace_back(e0, e1);
        if (collect)
            for (int i : idx)
                FPM_TRY(spectral_queue_collect(ctx, jobs[i], a, s, results[i].objects, results[i].object_spectra,
                                               b.launches));
        FPM_CUDA(cudaEventRecord(done, s));
        b.ends.push_back(done);
        if (k < 8) {
            b.st.bucket_size[k] = N;
            b.st.bucket_tiles[k] = (int32_t)idx.size();
            b.st.buckets = (int32_t)k + 1;
        }
        b.st.engine_bytes += bytes;
        b.groups.insert(b.groups.end(), idx.begin(), idx.end());
        ++k;
    }
    return Status::ok();
}

// After the queued work (and the result copies) have finished: status
// words, pass objectives and statistics from the recorded events.
Status spectral_finish(std::vector<SpectralJob>& jobs, const fpm_spectral_params* a,
                       const std::vector<fpm_spectral_result_desc>& results, SpectralBatch& b, fpm_run_stats& out) {
    for (size_t i = 0; i < jobs.size(); ++i) {
        if (jobs[i].host_status != 0)
            return Status::make(FPM_ERR_NUMERICAL, "problem %zu: device status %d", i, jobs[i].host_status);
        FPM_TRY(spectral_objectives(jobs[i], a, results[i].objectives));
    }
    fpm_run_stats st = b.st;
    double lo = 1e300, hi = -1e300;
    for (size_t g = 0; g < b.engine_events.size(); ++g) {
        float t0 = 0.f, t1 = 0.f, d = 0.f, end = 0.f;
        FPM_CUDA(cudaEventElapsedTime(&t0, b.start, b.engine_events[g].first));
        FPM_CUDA(cudaEventElapsedTime(&t1, b.start, b.engine_events[g].second));
        FPM_CUDA(cudaEventElapsedTime(&d, b.engine_events[g].first, b.engine_events[g].second));
        // run_ms and the group ends count from the inputs being resident
        // (after the measurement uploads), as for resident problems.
        FPM_CUDA(cudaEventElapsedTime(&end, b.uploaded, b.ends[g]));
        lo = std::min(lo, (double)t0);
        hi = std::max(hi, (double)t1);
        st.engine_ms_sum += d;
        st.run_ms = std::max(st.run_ms, (double)end);
        if (g < 8) st.bucket_end_ms[g] = end;
    }
    st.engine_span_ms = b.engine_events.empty() ? 0.0 : hi - lo;
    st.kernel_launches = b.launches;
    out = st;
    return Status::ok();
}

Status spectral_execute(fpm_context* ctx, std::vector<SpectralJob>& jobs, const fpm_spectral_params* a,
                        const std::vector<fpm_spectral_result_desc>& results) {
    FPM_CUDA(cudaSetDevice(ctx->device));
    const std::vector<cudaStream_t> streams(ctx->streams, ctx->streams + fpm_context::kStreams);
    SpectralBatch b;
    FPM_TRY(spectral_queue(ctx, jobs, a, results, streams, true, b));
    for (cudaStream_t s : streams) FPM_CUDA(cudaStreamSynchronize(s));
    FPM_CUDA(cudaGetLastError());
    return spectral_finish(jobs, a, results, b, ctx->stats);
}

Status spectral_run(fpm_context* ctx, const fpm_spectral_model_desc* sm, const fpm_measurement_desc* ms,
                    const fpm_spectral_params* a, const int32_t* order, const double* initial_objects,
                    const double* resume_spectra, int completed, double* objects_out, double* spectra_out,
                    double* objectives_out) {
    std::vector<SpectralJob> jobs(1);
    FPM_TRY(spectral_prepare(jobs[0], sm, ms, a, order, initial_objects, resume_spectra, completed));
    return spectral_execute(ctx, jobs, a, {fpm_spectral_result_desc{objects_out, spectra_out, objectives_out}});
}

Status spectral_run_batch(fpm_context* ctx, int count, const fpm_spectral_model_desc* models,
                          const fpm_measurement_desc* measurements, const fpm_spectral_params* a,
                          fpm_spectral_result_desc* results) {
    if (count <= 0 || !models || !measurements || !results)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "a positive problem count and its arrays are required");
    std::vector<SpectralJob> jobs(count);
    for (int i = 0; i < count; ++i) {
        Status st = spectral_prepare(jobs[i], &models[i], &measurements[i], a, nullptr, nullptr, nullptr, 0);
        if (st) return Status::make(st.code, "problem %d: %s", i, st.message.c_str());
    }
    return spectral_execute(ctx, jobs, a, std::vector<fpm_spectral_result_desc>(results, results + count));
}

}  // namespace

// A submitted batch: its buckets, device events and result destinations,
// completed by fpm_job_poll / fpm_job_wait.
struct fpm_job {
    fpm_context* ctx = nullptr;
    fpm_algorithm_params params{};
    fpm_result_desc* results = nullptr;
    std::vector<Bucket> buckets;
    std::vector<std::unique_ptr<BucketRun>> runs;
    // Spectral AP jobs instead of resident problems.
    bool spectral = false;
    fpm_spectral_params spectral_params{};
    std::vector<SpectralJob> spectral_jobs;
    std::vector<fpm_spectral_result_desc> spectral_results;
    std::unique_ptr<SpectralBatch> spectral_batch;
    std::vector<cudaStream_t> streams;
    cudaEvent_t done = nullptr;
    std::mutex mu;
    bool finished = false;
    Status status;
    fpm_run_stats stats{};
    ~fpm_job() {
        if (done) cudaEventSynchronize(done);
        for (cudaStream_t s : streams) cudaStreamSynchronize(s);
        // Buffers free on the job's streams before those are destroyed.
        runs.clear();
        spectral_batch.reset();
        spectral_jobs.clear();
        for (cudaStream_t s : streams) cudaStreamDestroy(s);
        if (done) cudaEventDestroy(done);
    }
};

namespace {

Status job_done_event(fpm_job* job);
Status create_job_streams(fpm_job* job, size_t count);

// fpm_run_batch without the wait: the buckets run on the job's own streams
// (jobs of one context overlap) and the results are copied as they finish.
Status submit_batch(fpm_context* ctx, int count, fpm_problem* const* problems, const fpm_algorithm_params* a,
                    fpm_result_desc* results, std::unique_ptr<fpm_job>& out) {
    FPM_TRY(validate_params(a));
    auto job = std::make_unique<fpm_job>();
    job->ctx = ctx;
    job->params = *a;
    job->results = results;
    FPM_TRY(build_buckets(ctx, count, problems, nullptr, job->buckets));
    FPM_TRY(create_job_streams(job.get(), job->buckets.size()));
    const size_t nstreams = job->streams.size();
    for (size_t k = 0; k < job->buckets.size(); ++k) {
        cudaStream_t s = job->streams[k % nstreams];
        job->runs.push_back(std::make_unique<BucketRun>());
        FPM_TRY(run_bucket(ctx, job->buckets[k], &job->params, s, *job->runs.back()));
    }
    FPM_TRY(job_done_event(job.get()));
    for (auto& b : job->buckets)
        for (fpm_problem* p : b.problems) p->busy = job.get();
    out = std::move(job);
    return Status::ok();
}

// Records the job's completion event behind every one of its streams.
Status job_done_event(fpm_job* job) {
    const size_t nstreams = job->streams.size();
    for (size_t k = 1; k < nstreams; ++k) {
        cudaEvent_t e;
        FPM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        const cudaError_t r1 = cudaEventRecord(e, job->streams[k]);
        const cudaError_t r2 = r1 == cudaSuccess ? cudaStreamWaitEvent(job->streams[0], e, 0) : r1;
        cudaEventDestroy(e);
        FPM_CUDA(r2);
    }
    FPM_CUDA(cudaEventCreateWithFlags(&job->done, cudaEventDisableTiming));
    FPM_CUDA(cudaEventRecord(job->done, job->streams[0]));
    return Status::ok();
}

Status create_job_streams(fpm_job* job, size_t count) {
    FPM_CUDA(cudaSetDevice(job->ctx->device));
    for (size_t k = 0; k < std::max<size_t>(1, std::min<size_t>(count, fpm_context::kStreams)); ++k) {
        cudaStream_t s;
        FPM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        job->streams.push_back(s);
    }
    return Status::ok();
}

// fpm_spectral_run_batch without the wait.
Status submit_spectral(fpm_context* ctx, int count, const fpm_spectral_model_desc* models,
                       const fpm_measurement_desc* measurements, const fpm_spectral_params* a,
                       fpm_spectral_result_desc* results, std::unique_ptr<fpm_job>& out) {
    if (count <= 0 || !models || !measurements || !results || !a)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "a positive problem count and its arrays are required");
    auto job = std::make_unique<fpm_job>();
    job->ctx = ctx;
    job->spectral = true;
    job->spectral_params = *a;
    job->spectral_jobs = std::vector<SpectralJob>(count);
    job->spectral_results.assign(results, results + count);
    for (int i = 0; i < count; ++i) {
        Status st = spectral_prepare(job->spectral_jobs[i], &models[i], &measurements[i], &job->spectral_params,
                                     nullptr, nullptr, nullptr, 0);
        if (st) return Status::make(st.code, "problem %d: %s", i, st.message.c_str());
    }
    std::map<int, int> sizes;
    for (auto& j : job->spectral_jobs) sizes[j.N] = 1;
    FPM_TRY(create_job_streams(job.get(), sizes.size()));
    job->spectral_batch = std::make_unique<SpectralBatch>();
    FPM_TRY(spectral_queue(ctx, job->spectral_jobs, &job->spectral_params, job->spectral_results, job->streams, false,
                           *job->spectral_batch));
    FPM_TRY(job_done_event(job.get()));
    out = std::move(job);
    return Status::ok();
}

// Runs once, after the job's completion event: status words, objectives
// and statistics; the problems' buffers return to a context stream and the
// problems become usable again.
// Result downloads go to pageable caller memory, which makes a copy wait
// for its stream; they are therefore queued here, after the device work,
// and waited for at once.
Status collect_job(fpm_job* j) {
    cudaStream_t s = j->streams[0];
    if (j->spectral) {
        for (size_t i = 0; i < j->spectral_jobs.size(); ++i)
            FPM_TRY(spectral_queue_collect(j->ctx, j->spectral_jobs[i], &j->spectral_params, s,
                                           j->spectral_results[i].objects, j->spectral_results[i].object_spectra,
                                           j->spectral_batch->launches));
    } else {
        for (auto& b : j->buckets)
            for (size_t t = 0; t < b.problems.size(); ++t)
                FPM_TRY(queue_collect(b.problems[t], &j->params, j->results ? &j->results[b.indices[t]] : nullptr, s));
    }
    FPM_CUDA(cudaStreamSynchronize(s));
    FPM_CUDA(cudaGetLastError());
    if (j->spectral)
        return spectral_finish(j->spectral_jobs, &j->spectral_params, j->spectral_results, *j->spectral_batch, j->stats);
    for (auto& b : j->buckets)
        for (size_t t = 0; t < b.problems.size(); ++t) {
            Status s2 = finish_collect(b.problems[t], &j->params, j->results ? &j->results[b.indices[t]] : nullptr);
            if (s2) return Status::make(s2.code, "problem %d: %s", b.indices[t], s2.message.c_str());
        }
    return compute_stats(j->buckets, j->runs, j->stats);
}

void finish_job(fpm_job* j) {
    std::lock_guard<std::mutex> lock(j->ctx->mu);
    cudaSetDevice(j->ctx->device);
    j->status = collect_job(j);
    for (auto& b : j->buckets)
        for (fpm_problem* p : b.problems) {
            for (DeviceBuffer* buf : run_buffers(p)) buf->bind(j->ctx->pool, j->ctx->streams[0]);
            p->busy = nullptr;
        }
    j->finished = true;
}
}  // namespace

// A captured run plan: the device work of one run_batch over resident
// problems (initialisation, frame engine, per-iteration gauge, regulariser
// and illumination steps, finalisation, for every tile size on its own
// stream) recorded once as a CUDA graph and replayed as one launch. Each
// replay starts from the problems' initial state, exactly as a fresh run.
struct fpm_plan {
    fpm_context* ctx = nullptr;
    fpm_algorithm_params params{};
    std::vector<Bucket> buckets;
    std::vector<std::unique_ptr<BucketRun>> runs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int streams = 0;
    ~fpm_plan() {
        if (ctx)
            for (int k = 0; k < streams; ++k) cudaStreamSynchronize(ctx->streams[k]);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto& b : buckets)
            for (fpm_problem* p : b.problems) p->plan = nullptr;
        runs.clear();  // buffers free on their streams
    }
};

namespace {

Status plan_create(fpm_context* ctx, int count, fpm_problem* const* problems, const fpm_algorithm_params* a,
                   std::unique_ptr<fpm_plan>& out) {
    FPM_TRY(validate_params(a));
    auto plan = std::make_unique<fpm_plan>();
    plan->ctx = ctx;
    plan->params = *a;
    FPM_TRY(build_buckets(ctx, count, problems, nullptr, plan->buckets));
    const int ns = (int)std::min<size_t>(plan->buckets.size(), fpm_context::kStreams);
    plan->streams = ns;
    // Host preparation: buffers, descriptor tables and FFT plans.
    for (size_t k = 0; k < plan->buckets.size(); ++k) {
        plan->runs.push_back(std::make_unique<BucketRun>());
        BucketRun& br = *plan->runs.back();
        br.launch = false;
        FPM_TRY(run_bucket(ctx, plan->buckets[k], &plan->params, ctx->streams[k % fpm_context::kStreams], br));
    }
    for (int k = 0; k < ns; ++k) FPM_CUDA(cudaStreamSynchronize(ctx->streams[k]));
    // Capture: the first stream forks to the others and joins them at the end.
    cudaStream_t s0 = ctx->streams[0];
    FPM_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
    std::vector<cudaEvent_t> marks;
    auto captured = [&]() -> Status {
        cudaEvent_t fork;
        FPM_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        marks.push_back(fork);
        FPM_CUDA(cudaEventRecord(fork, s0));
        for (int k = 1; k < ns; ++k) FPM_CUDA(cudaStreamWaitEvent(ctx->streams[k], fork, 0));
        for (size_t k = 0; k < plan->buckets.size(); ++k) {
            BucketRun& br = *plan->runs[k];
            br.prepare = false;
            br.launch = true;
            br.captured = true;
            FPM_TRY(run_bucket(ctx, plan->buckets[k], &plan->params, ctx->streams[k % fpm_context::kStreams], br));
        }
        for (int k = 1; k < ns; ++k) {
            cudaEvent_t join;
            FPM_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
            marks.push_back(join);
            FPM_CUDA(cudaEventRecord(join, ctx->streams[k]));
            FPM_CUDA(cudaStreamWaitEvent(s0, join, 0));
        }
        return Status::ok();
    };
    Status st = captured();
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(s0, &graph);
    for (cudaEvent_t e : marks) cudaEventDestroy(e);
    if (st) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    FPM_CUDA(end);
    plan->graph = graph;
    FPM_CUDA(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
    for (auto& b : plan->buckets)
        for (fpm_problem* p : b.problems) p->plan = plan.get();
    out = std::move(plan);
    return Status::ok();
}

}  // namespace

namespace fpm {

void set_context_error(fpm_context* ctx, const char* message) {
    if (ctx) ctx->error = message;
    g_global_error = message;
}

void context_device_stream(fpm_context* ctx, int* device, cudaStream_t* stream) {
    *device = ctx->device;
    *stream = ctx->streams[0];
}

std::mutex& context_mutex(fpm_context* ctx) { return ctx->mu; }

}  // namespace fpm

// ====================================================================== ABI

namespace {

// Forward intensity stack into the device buffer `out` (float, F*N*N).
// `object` is the natural-order object, or with `centred` its centred
// spectrum (the state of a reconstruction).
Status forward_stack_device(fpm_context* ctx, const fpm_model_desc* md, const double* object, DeviceBuffer& out,
                            cudaStream_t s, bool centred = false) {
        FPM_TRY(validate_model(md));
        if (!object) return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        const int N = md->image_height, M = md->recon_height, F = md->sources;
        if (md->image_width != N || !fpm::engine_supported(N) || md->recon_width != M)
            return Status::make(FPM_ERR_UNSUPPORTED,
                                "the GB300 device path supports square detector frames of 32, 64, 128 or 256 pixels");
        FPM_CUDA(cudaSetDevice(ctx->device));
        const size_t n2 = (size_t)N * N, m2 = (size_t)M * M;
        const long long ms = M + (M & 1);
        // Frame constants (gains, stencils) as for a problem without masks.
        std::vector<fpm::FrameParam> params(F);
        for (int f = 0; f < F; ++f) {
            Axis r{}, c{};
            const double orow = md->offset_row ? md->offset_row[f] : 0.0, ocol = md->offset_col ? md->offset_col[f] : 0.0;
            FPM_TRY(interpolation_axis(md->crop_start_row[f], N, M, orow, r));
            FPM_TRY(interpolation_axis(md->crop_start_col[f], N, M, ocol, c));
            fpm::FrameParam fp{};
            const bool zero = std::fabs(orow) <= 1e-12 && std::fabs(ocol) <= 1e-12;
            fp.lower_row = zero ? (int)md->crop_start_row[f] : (int)r.lower_start;
            fp.lower_col = zero ? (int)md->crop_start_col[f] : (int)c.lower_start;
            fp.has_upper_row = zero ? 0 : (r.upper ? 1 : 0);
            fp.has_upper_col = zero ? 0 : (c.upper ? 1 : 0);
            fp.w00 = zero ? 1.f : (float)(r.lower_weight * c.lower_weight);
            fp.w01 = zero ? 0.f : (float)(r.lower_weight * c.upper_weight);
            fp.w10 = zero ? 0.f : (float)(r.upper_weight * c.lower_weight);
            fp.w11 = zero ? 0.f : (float)(r.upper_weight * c.upper_weight);
            const double g = md->frame_gains ? md->frame_gains[f] : 1.0;
            if (!(g > 0.0)) return Status::make(FPM_ERR_INVALID_MODEL, "frame %d has invalid gain %g", f, g);
            fp.gain = (float)g;
            fp.weight = 1.f;
            params[f] = fp;
        }
        DeviceBuffer d_params, d_pupil, d_obj64, d_state, d_ptrs, d_ptrs2, d_bg;
        FPM_TRY(upload_array(ctx, d_params, params, s));
        std::vector<float2> pf(n2);
        for (size_t i = 0; i < n2; ++i) pf[i] = make_float2((float)md->pupil[2 * i], (float)md->pupil[2 * i + 1]);
        FPM_TRY(upload_array(ctx, d_pupil, pf, s));
        FPM_TRY(d_obj64.ensure(sizeof(double2) * m2));
        FPM_CUDA(cudaMemcpyAsync(d_obj64.ptr, object, sizeof(double2) * m2, cudaMemcpyHostToDevice, s));
        FPM_TRY(d_state.ensure(sizeof(float2) * (size_t)M * ms));
        std::vector<double2*> p64 = {d_obj64.as<double2>()};
        std::vector<float2*> pst = {d_state.as<float2>()};
        FPM_TRY(upload_array(ctx, d_ptrs, p64, s));
        FPM_TRY(upload_array(ctx, d_ptrs2, pst, s));
        if (centred) {
            FPM_CUDA(fpm::launch_narrow(d_obj64.as<double2>(), M, M, d_state.as<float2>(), ms, s));
        } else {
            // object_spectrum (src/simulation/simulator.rs:209-226): forward FFT, fftshift.
            FPM_TRY(fft2_device(ctx, d_ptrs.as<double2*>(), 1, M, M, false, s));
            FPM_CUDA(fpm::launch_shift_to_state(d_ptrs.as<double2*>(), d_ptrs2.as<float2*>(), nullptr, nullptr, 1, M, s));
        }
        fpm::ForwardParams fwd{};
        fwd.object = d_state.as<float2>();
        fwd.pupil = d_pupil.as<float2>();
        fwd.params = d_params.as<fpm::FrameParam>();
        if (md->background) {
            std::vector<float> bg(md->background, md->background + md->background_len);
            FPM_TRY(upload_array(ctx, d_bg, bg, s));
            fwd.background = d_bg.as<float>();
            fwd.background_stride = md->background_len == (int64_t)n2 ? 0 : (long long)n2;
        }
        FPM_TRY(out.ensure(sizeof(float) * n2 * F));
        fwd.out = out.as<float>();
        fwd.M = M;
        fwd.frame_count = F;
        FPM_CUDA(fpm::launch_forward(N, fwd, s));
        // The temporaries above are freed on return: wait for the kernels that use them.
        FPM_CUDA(cudaStreamSynchronize(s));
        return Status::ok();
}

Status validate_camera(const fpm_camera_desc* c, size_t frame_len) {
    if (!c) return Status::ok();
    auto bad = [](double v) { return !std::isfinite(v) || v < 0.0; };
    if (!std::isfinite(c->photons_per_pixel) || c->photons_per_pixel <= 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "photons_per_pixel must be finite and positive");
    if (!std::isfinite(c->gain_counts_per_electron) || c->gain_counts_per_electron <= 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "gain_counts_per_electron must be finite and positive");
    if (!std::isfinite(c->offset_counts) || bad(c->read_noise_electrons) || bad(c->dark_current_electrons))
        return Status::make(FPM_ERR_INVALID_PARAMETER, "offset, read noise and dark current must be finite (noise and dark current non-negative)");
    if (std::isnan(c->maximum_count) || c->maximum_count < 0.0)
        return Status::make(FPM_ERR_INVALID_PARAMETER, "maximum_count must be non-negative");
    if (c->pixel_sensitivity)
        for (size_t i = 0; i < frame_len; ++i)
            if (bad(c->pixel_sensitivity[i]))
                return Status::make(FPM_ERR_INVALID_PARAMETER, "pixel_sensitivity must be finite and non-negative");
    if (c->bad_pixel_count < 0 || (c->bad_pixel_count > 0 && !c->bad_pixels))
        return Status::make(FPM_ERR_INVALID_PARAMETER, "bad pixel list is invalid");
    for (int64_t k = 0; k < c->bad_pixel_count; ++k)
        if (c->bad_pixels[k] < 0 || (size_t)c->bad_pixels[k] >= frame_len)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "bad_pixels indices must be below the frame size %zu", frame_len);
    return Status::ok();
}

}  // namespace

extern "C" {

const char* fpm_global_last_error(void) { return g_global_error.c_str(); }

int32_t fpm_create(fpm_context** out, int32_t device) {
    if (!out) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "output pointer is null"));
    auto ctx = std::make_unique<fpm_context>();
    ctx->device = device;
    auto init = [&]() -> Status {
        int count = 0;
        FPM_CUDA(cudaGetDeviceCount(&count));
        if (device < 0 || device >= count)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "device %d is not available (%d devices)", device, count);
        FPM_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop{};
        FPM_CUDA(cudaGetDeviceProperties(&prop, device));
        if (prop.major < 10)
            return Status::make(FPM_ERR_UNSUPPORTED, "device %d (%s, sm_%d%d) is not a Blackwell GPU; this library targets sm_103a",
                                device, prop.name, prop.major, prop.minor);
        for (int i = 0; i < fpm_context::kStreams; ++i)
            FPM_CUDA(cudaStreamCreateWithFlags(&ctx->streams[i], cudaStreamNonBlocking));
        FPM_CUDA(cudaStreamCreateWithFlags(&ctx->upload, cudaStreamNonBlocking));
        FPM_CUDA(cudaStreamCreateWithFlags(&ctx->download, cudaStreamNonBlocking));
        // Problem buffers come from a private stream-ordered pool that keeps
        // freed memory for the next problems instead of returning it.
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        FPM_CUDA(cudaMemPoolCreate(&ctx->pool, &props));
        uint64_t threshold = ~0ull;
        FPM_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &threshold));
        return Status::ok();
    };
    Status s = init();
    if (s) return finish(nullptr, s);
    *out = ctx.release();
    return FPM_OK;
}

int32_t fpm_destroy(fpm_context* ctx) {
    if (!ctx) return FPM_OK;
    cudaSetDevice(ctx->device);
    for (int i = 0; i < fpm_context::kStreams; ++i)
        if (ctx->streams[i]) cudaStreamSynchronize(ctx->streams[i]);
    for (cudaStream_t extra : {ctx->upload, ctx->download})
        if (extra) cudaStreamSynchronize(extra);
    for (int i = 0; i < fpm_context::kStreams; ++i)
        if (ctx->streams[i]) cudaStreamDestroy(ctx->streams[i]);
    for (cudaStream_t extra : {ctx->upload, ctx->download})
        if (extra) cudaStreamDestroy(extra);
    // Outstanding pooled allocations (problems not yet destroyed) keep the
    // pool's memory until they are freed.
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    delete ctx;
    return FPM_OK;
}

int32_t fpm_last_error(const fpm_context* ctx, char* buffer, size_t length) {
    if (!buffer || length == 0) return FPM_ERR_INVALID_PARAMETER;
    const std::string& msg = ctx ? ctx->error : g_global_error;
    std::snprintf(buffer, length, "%s", msg.c_str());
    return FPM_OK;
}

int32_t fpm_planar_led_kvectors(const fpm_optics* optics, int32_t rows, int32_t cols, double pitch_x, double pitch_y,
                                double reference_col, double reference_row, const double* translation,
                                const double* rotation_rad, double* kx, double* ky) {
    auto body = [&]() -> Status {
        if (!optics || !translation || !rotation_rad || !kx || !ky)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        FPM_TRY(validate_optics(*optics));
        if (rows <= 0 || cols <= 0) return Status::make(FPM_ERR_INVALID_PARAMETER, "shape rows and columns must be non-zero");
        if (!std::isfinite(pitch_x) || !std::isfinite(pitch_y) || pitch_x <= 0.0 || pitch_y <= 0.0)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "pitch_x and pitch_y must be finite and positive");
        const double k = 2.0 * M_PI * optics->illumination_refractive_index / optics->wavelength_vacuum_m;
        const double sx = std::sin(rotation_rad[0]), cx = std::cos(rotation_rad[0]);
        const double sy = std::sin(rotation_rad[1]), cy = std::cos(rotation_rad[1]);
        const double sz = std::sin(rotation_rad[2]), cz = std::cos(rotation_rad[2]);
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c) {
                const double p[3] = {((double)c - reference_col) * pitch_x, ((double)r - reference_row) * pitch_y, 0.0};
                const double ax[3] = {p[0], cx * p[1] - sx * p[2], sx * p[1] + cx * p[2]};
                const double ay[3] = {cy * ax[0] + sy * ax[2], ax[1], -sy * ax[0] + cy * ax[2]};
                const double az[3] = {cz * ay[0] - sz * ay[1], sz * ay[0] + cz * ay[1], ay[2]};
                const double pos[3] = {az[0] + translation[0], az[1] + translation[1], az[2] + translation[2]};
                const double norm = std::hypot(std::hypot(pos[0], pos[1]), pos[2]);
                if (!std::isfinite(norm) || norm <= 0.0)
                    return Status::make(FPM_ERR_INVALID_PARAMETER, "no source may coincide with the sample origin");
                kx[r * cols + c] = k * (-pos[0] / norm);
                ky[r * cols + c] = k * (-pos[1] / norm);
            }
        return Status::ok();
    };
    return finish(nullptr, body());
}

// The objective's data term on host intensities (loss and point_loss,
// src/algorithms/objective.rs:27-72): per-value losses summed in order in
// FP64, then divided by the count. Amplitude, Poisson and Huber losses clamp
// negative intensities to zero.
int32_t fpm_intensity_loss(const double* predicted, const double* measured, int64_t count, int32_t loss_type,
                           double* out) {
    auto body = [&]() -> Status {
        if (!predicted || !measured || !out) return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        if (loss_type < FPM_LOSS_AMPLITUDE_MSE || loss_type > FPM_LOSS_HUBER_AMPLITUDE)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "unknown loss_type %d", loss_type);
        if (count <= 0)
            return Status::make(FPM_ERR_INVALID_SHAPE, "loss inputs have lengths %lld and %lld", (long long)count,
                                (long long)count);
        double sum = 0.0;
        for (int64_t i = 0; i < count; ++i) {
            const double p = predicted[i], m = measured[i];
            if (!std::isfinite(p) || !std::isfinite(m))
                return Status::make(FPM_ERR_NUMERICAL, "loss input contains a non-finite value");
            double term;
            if (loss_type == FPM_LOSS_INTENSITY_MSE) {
                const double r = p - m;
                term = r * r;
            } else if (loss_type == FPM_LOSS_POISSON_NLL) {
                const double mean = std::max(p, 1e-12);
                term = mean - std::max(m, 0.0) * std::log(mean);
            } else {
                const double r = std::sqrt(std::max(p, 0.0)) - std::sqrt(std::max(m, 0.0));
                if (loss_type == FPM_LOSS_AMPLITUDE_MSE)
                    term = r * r;
                else
                    term = std::fabs(r) <= 1.0 ? 0.5 * r * r : std::fabs(r) - 0.5;
            }
            sum += term;
        }
        *out = sum / (double)count;
        return Status::ok();
    };
    return finish(nullptr, body());
}

int32_t fpm_suggest_shape(const fpm_optics* optics, int32_t sources, const double* kx, const double* ky,
                          int32_t image_height, int32_t image_width, int32_t policy, int32_t* recon_height,
                          int32_t* recon_width) {
    auto body = [&]() -> Status {
        if (!optics || !kx || !ky || !recon_height || !recon_width)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        FPM_TRY(validate_optics(*optics));
        Bounds b{};
        FPM_TRY(displacement_bounds(*optics, sources, kx, ky, image_height, image_width, b));
        int mh = *recon_height, mw = *recon_width;
        FPM_TRY(resolve_shape(image_height, image_width, policy, mh, mw, b));
        *recon_height = mh;
        *recon_width = mw;
        return Status::ok();
    };
    return finish(nullptr, body());
}

int32_t fpm_compile_model(const fpm_optics* optics, int32_t sources, const double* kx, const double* ky,
                          int32_t h, int32_t w, int32_t policy, int32_t* recon_height, int32_t* recon_width,
                          int64_t* start_row, int64_t* start_col, double* offset_row, double* offset_col,
                          double* pupil, uint8_t* support, double* dkx_out, double* dky_out) {
    auto body = [&]() -> Status {
        if (!optics || !kx || !ky || !recon_height || !recon_width || !start_row || !start_col || !offset_row ||
            !offset_col || !pupil || !support)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        FPM_TRY(validate_optics(*optics));
        for (int s = 0; s < sources; ++s)
            if (!std::isfinite(kx[s]) || !std::isfinite(ky[s]))
                return Status::make(FPM_ERR_INVALID_MODEL, "k-vectors must contain finite values");
        Bounds b{};
        FPM_TRY(displacement_bounds(*optics, sources, kx, ky, h, w, b));
        int mh = *recon_height, mw = *recon_width;
        FPM_TRY(resolve_shape(h, w, policy, mh, mw, b));
        const double low = optics->camera_pixel_size / optics->magnification;
        const double dkx = 2.0 * M_PI / ((double)w * low), dky = 2.0 * M_PI / ((double)h * low);
        // Pupil::circular (src/model/pupil.rs:78-123).
        const double cutoff = 2.0 * M_PI * optics->objective_na / optics->wavelength_vacuum_m;
        const double medium_k = 2.0 * M_PI * optics->objective_medium_refractive_index / optics->wavelength_vacuum_m;
        for (int r = 0; r < h; ++r) {
            const double y = ((double)r - (double)(h / 2)) * dky;
            for (int c = 0; c < w; ++c) {
                const double x = ((double)c - (double)(w / 2)) * dkx;
                const double radius = std::hypot(x, y);
                const size_t i = (size_t)r * w + c;
                const bool inside = radius <= cutoff;
                support[i] = inside ? 1 : 0;
                if (!inside) {
                    pupil[2 * i] = pupil[2 * i + 1] = 0.0;
                    continue;
                }
                const double rho = cutoff > 0.0 ? radius / cutoff : 0.0;
                const double theta = std::atan2(y, x);
                double phase = 0.0, amplitude = 1.0;
                if (optics->has_defocus) phase -= optics->defocus_distance * (x * x + y * y) / (2.0 * medium_k);
                if (optics->has_aberration) {
                    phase += optics->astigmatism * rho * rho * std::cos(2.0 * theta);
                    phase += optics->coma * (3.0 * std::pow(rho, 3) - 2.0 * rho) * std::cos(theta);
                    phase += optics->spherical * (6.0 * std::pow(rho, 4) - 6.0 * rho * rho + 1.0);
                    amplitude = std::exp(-optics->edge_apodization * rho * rho);
                }
                pupil[2 * i] = amplitude * std::cos(phase);
                pupil[2 * i + 1] = amplitude * std::sin(phase);
            }
        }
        // crop_for_k_vector (src/model/image_plane_fpm.rs:750-797).
        for (int s = 0; s < sources; ++s) {
            GridShift row{}, col{};
            FPM_TRY(grid_shift(ky[s] / dky, row));
            FPM_TRY(grid_shift(kx[s] / dkx, col));
            const long long sr = mh / 2 - h / 2 + row.integer, sc = mw / 2 - w / 2 + col.integer;
            if (sr < 0 || sc < 0)
                return Status::make(FPM_ERR_INVALID_MODEL, "illumination vector %d produces a crop outside the reconstruction grid", s);
            Axis a{};
            FPM_TRY(interpolation_axis(sr, h, mh, row.offset, a));
            FPM_TRY(interpolation_axis(sc, w, mw, col.offset, a));
            start_row[s] = sr;
            start_col[s] = sc;
            offset_row[s] = row.offset;
            offset_col[s] = col.offset;
        }
        *recon_height = mh;
        *recon_width = mw;
        if (dkx_out) *dkx_out = dkx;
        if (dky_out) *dky_out = dky;
        return Status::ok();
    };
    return finish(nullptr, body());
}

int32_t fpm_fft2(fpm_context* ctx, double* values, int32_t height, int32_t width, int32_t inverse) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        if (!values) return Status::make(FPM_ERR_INVALID_PARAMETER, "values is null");
        if (height <= 0 || width <= 0) return Status::make(FPM_ERR_INVALID_SHAPE, "FFT dimensions must be non-zero");
        FPM_CUDA(cudaSetDevice(ctx->device));
        cudaStream_t s = ctx->streams[0];
        const size_t bytes = sizeof(double2) * (size_t)height * width;
        FPM_TRY(ctx->scratch_a.ensure(bytes));
        FPM_TRY(ctx->scratch_b.ensure(sizeof(double2*)));
        double2* arr = ctx->scratch_a.as<double2>();
        FPM_CUDA(cudaMemcpyAsync(ctx->scratch_b.ptr, &arr, sizeof(double2*), cudaMemcpyHostToDevice, s));
        FPM_CUDA(cudaMemcpyAsync(arr, values, bytes, cudaMemcpyHostToDevice, s));
        FPM_TRY(fft2_device(ctx, ctx->scratch_b.as<double2*>(), 1, height, width, inverse != 0, s));
        FPM_CUDA(cudaMemcpyAsync(values, arr, bytes, cudaMemcpyDeviceToHost, s));
        FPM_CUDA(cudaStreamSynchronize(s));
        return Status::ok();
    };
    return finish(ctx, body());
}


int32_t fpm_forward_stack(fpm_context* ctx, const fpm_model_desc* md, const double* object, double* intensities) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        if (!intensities) return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        FPM_TRY(validate_model(md));
        cudaStream_t s = ctx->streams[0];
        DeviceBuffer d_out;
        FPM_TRY(forward_stack_device(ctx, md, object, d_out, s));
        const size_t total = (size_t)md->image_height * md->image_width * md->sources;
        std::vector<float> host(total);
        FPM_CUDA(cudaMemcpyAsync(host.data(), d_out.ptr, sizeof(float) * total, cudaMemcpyDeviceToHost, s));
        FPM_CUDA(cudaStreamSynchronize(s));
        for (size_t i = 0; i < total; ++i) intensities[i] = host[i];
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_simulate_stack(fpm_context* ctx, const fpm_model_desc* md, const double* object,
                           const fpm_camera_desc* camera, uint64_t seed, double* counts) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        if (!counts) return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        FPM_TRY(validate_model(md));
        const size_t frame_len = (size_t)md->image_height * md->image_width;
        FPM_TRY(validate_camera(camera, frame_len));
        const size_t total = frame_len * md->sources;
        cudaStream_t s = ctx->streams[0];
        DeviceBuffer d_out, d_counts, d_sens, d_status;
        FPM_TRY(forward_stack_device(ctx, md, object, d_out, s));
        fpm::CameraParams cp{};
        if (camera) {
            cp.photons_per_pixel = camera->photons_per_pixel;
            cp.gain_counts_per_electron = camera->gain_counts_per_electron;
            cp.offset_counts = camera->offset_counts;
            cp.read_noise = camera->read_noise_electrons;
            cp.dark_current = camera->dark_current_electrons;
            cp.maximum_count = camera->maximum_count;
            cp.shot_noise = camera->shot_noise;
            cp.quantize = camera->quantize;
            if (camera->pixel_sensitivity) {
                FPM_TRY(d_sens.ensure(sizeof(double) * frame_len));
                FPM_CUDA(cudaMemcpyAsync(d_sens.ptr, camera->pixel_sensitivity, sizeof(double) * frame_len,
                                         cudaMemcpyHostToDevice, s));
                cp.sensitivity = d_sens.as<double>();
            }
        } else {
            // No camera: the intensities themselves (CameraModel::ideal).
            cp.photons_per_pixel = 1.0;
            cp.gain_counts_per_electron = 1.0;
            cp.maximum_count = INFINITY;
        }
        cp.seed = seed;
        FPM_TRY(d_counts.ensure(sizeof(double) * total));
        FPM_TRY(d_status.ensure(sizeof(int)));
        FPM_CUDA(cudaMemsetAsync(d_status.ptr, 0, sizeof(int), s));
        FPM_CUDA(fpm::launch_camera(d_out.as<float>(), d_counts.as<double>(), (long long)total, (long long)frame_len, cp,
                                    d_status.as<int>(), s));
        int status = 0;
        FPM_CUDA(cudaMemcpyAsync(counts, d_counts.ptr, sizeof(double) * total, cudaMemcpyDeviceToHost, s));
        FPM_CUDA(cudaMemcpyAsync(&status, d_status.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
        FPM_CUDA(cudaStreamSynchronize(s));
        if (status) return Status::make(FPM_ERR_NUMERICAL, "a Poisson draw did not terminate within its bound");
        if (camera && camera->bad_pixel_count > 0) {
            double value = std::isnan(camera->bad_pixel_value) ? camera->maximum_count : camera->bad_pixel_value;
            value = std::min(std::max(value, 0.0), camera->maximum_count);
            if (camera->quantize) value = std::round(value);
            for (int f = 0; f < md->sources; ++f)
                for (int64_t k = 0; k < camera->bad_pixel_count; ++k) counts[(size_t)f * frame_len + camera->bad_pixels[k]] = value;
        }
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_problem_create(fpm_context* ctx, const fpm_model_desc* model, const fpm_measurement_desc* measurements,
                           fpm_problem** problem) {
    if (!ctx || !problem) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    return finish(ctx, create_problem(ctx, model, measurements, problem));
}

int32_t fpm_problem_create_batch(fpm_context* ctx, int32_t count, const fpm_model_desc* models,
                                 const fpm_measurement_desc* measurements, fpm_problem** problems) {
    if (!ctx || count < 0 || (count > 0 && (!models || !measurements || !problems)))
        return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument or negative count"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    for (int i = 0; i < count; ++i) problems[i] = nullptr;
    std::vector<std::unique_ptr<fpm_problem>> made;
    Status s = create_problems(ctx, count, models, measurements, made);
    if (s) {
        made.clear();
        return finish(ctx, s);
    }
    for (int i = 0; i < count; ++i) problems[i] = made[i].release();
    return finish(ctx, s);
}

int32_t fpm_problem_destroy(fpm_problem* problem) {
    if (!problem) return FPM_OK;
    fpm_context* ctx = problem->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (problem->busy)
        return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "the problem is in use by a submitted job"));
    if (problem->plan)
        return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "the problem is held by a captured run plan"));
    cudaSetDevice(ctx->device);
    delete problem;
    return FPM_OK;
}

int32_t fpm_run(fpm_context* ctx, fpm_problem* problem, const fpm_algorithm_params* params, fpm_result_desc* result) {
    return fpm_run_batch(ctx, 1, &problem, params, result);
}

int32_t fpm_run_batch(fpm_context* ctx, int32_t count, fpm_problem* const* problems, const fpm_algorithm_params* params,
                      fpm_result_desc* results) {
    if (!ctx || (count > 0 && !problems)) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    return finish(ctx, run_batch(ctx, count, problems, params, results));
}

int32_t fpm_run_batch_resumable(fpm_context* ctx, int32_t count, fpm_problem* const* problems,
                                const fpm_algorithm_params* params, const fpm_state_desc* resume,
                                fpm_result_desc* results, fpm_state_desc* capture) {
    if (!ctx || (count > 0 && !problems)) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    return finish(ctx, run_batch(ctx, count, problems, params, results, resume, capture));
}

int32_t fpm_run_batch_host(fpm_context* ctx, int32_t count, const fpm_model_desc* models,
                           const fpm_measurement_desc* measurements, const fpm_algorithm_params* params,
                           fpm_result_desc* results, fpm_problem** problems) {
    if (!ctx || count < 0 || (count > 0 && (!models || !measurements || !problems)))
        return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument or negative count"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    for (int i = 0; i < count; ++i) problems[i] = nullptr;
    std::vector<std::unique_ptr<fpm_problem>> made;
    Status s = run_batch_host(ctx, count, models, measurements, params, results, made);
    if (s) {
        // Work already queued must finish before its buffers are released.
        for (int i = 0; i < fpm_context::kStreams; ++i) cudaStreamSynchronize(ctx->streams[i]);
        cudaStreamSynchronize(ctx->upload);
        cudaStreamSynchronize(ctx->download);
        made.clear();
        return finish(ctx, s);
    }
    for (int i = 0; i < count; ++i) problems[i] = made[i].release();
    return finish(ctx, s);
}

int32_t fpm_spectral_run(fpm_context* ctx, const fpm_spectral_model_desc* model,
                         const fpm_measurement_desc* measurements, const fpm_spectral_params* params,
                         const int32_t* order, const double* initial_objects, const double* resume_spectra,
                         int32_t completed_iterations, double* objects, double* object_spectra, double* objectives) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    return finish(ctx, spectral_run(ctx, model, measurements, params, order, initial_objects, resume_spectra,
                                    completed_iterations, objects, object_spectra, objectives));
}

int32_t fpm_spectral_run_batch(fpm_context* ctx, int32_t count, const fpm_spectral_model_desc* models,
                               const fpm_measurement_desc* measurements, const fpm_spectral_params* params,
                               fpm_spectral_result_desc* results) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    return finish(ctx, spectral_run_batch(ctx, count, models, measurements, params, results));
}

int32_t fpm_spectral_forward(fpm_context* ctx, const fpm_spectral_model_desc* model, const double* spectra,
                             double* intensities) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        if (!model || !spectra || !intensities) return Status::make(FPM_ERR_INVALID_PARAMETER, "null argument");
        fpm_measurement_desc none{};
        if (model->channels <= 0 || !model->channel_models)
            return Status::make(FPM_ERR_INVALID_PARAMETER, "at least one spectral channel is required");
        const fpm_model_desc& c0 = model->channel_models[0];
        const size_t n2 = (size_t)c0.image_height * c0.image_width, nm = (size_t)c0.recon_height * c0.recon_width;
        // Model checks only: a stand-in measurement header of the right frame count.
        std::vector<double> zeros;
        none.frames = model->exposures;
        zeros.assign(n2 * (size_t)std::max(model->exposures, 0), 1.0);
        none.measurements = zeros.data();
        fpm_spectral_params prm{1, 1, 0, 1.0, 1e-10};
        FPM_TRY(validate_spectral(model, &none, &prm));
        const size_t objects = model->object_coupling == FPM_COUPLING_SHARED_COMPLEX ? 1 : (size_t)model->channels;
        for (size_t i = 0; i < 2 * nm * objects; ++i)
            if (!std::isfinite(spectra[i])) return Status::make(FPM_ERR_INVALID_PARAMETER, "complex values must be finite");
        cudaStream_t s = ctx->streams[0];
        std::vector<double> out(n2 * model->exposures, 0.0);
        std::vector<float> local;
        for (int c = 0; c < model->channels; ++c) {
            const fpm_model_desc& md = model->channel_models[c];
            const size_t o = model->object_coupling == FPM_COUPLING_SHARED_COMPLEX ? 0 : (size_t)c;
            DeviceBuffer d_out;
            FPM_TRY(forward_stack_device(ctx, &md, spectra + 2 * nm * o, d_out, s, true));
            local.resize(n2 * md.sources);
            FPM_CUDA(cudaMemcpyAsync(local.data(), d_out.ptr, sizeof(float) * local.size(), cudaMemcpyDeviceToHost, s));
            FPM_CUDA(cudaStreamSynchronize(s));
            // gain[f] * sum_k w_k * local_k + background[f]
            // (SpectralImagePlaneModel::forward_intensity, src/model/spectral.rs:400-446).
            for (int e = 0; e < model->exposures; ++e)
                for (int k = model->contribution_offsets[e]; k < model->contribution_offsets[e + 1]; ++k) {
                    if (model->contribution_channel[k] != c) continue;
                    const double w = model->contribution_weight[k];
                    const float* src = local.data() + n2 * model->contribution_local_frame[k];
                    double* dst = out.data() + n2 * e;
                    for (size_t i = 0; i < n2; ++i) dst[i] += w * (double)src[i];
                }
        }
        for (int e = 0; e < model->exposures; ++e)
            for (size_t i = 0; i < n2; ++i)
                intensities[n2 * e + i] = model->exposure_gain[e] * out[n2 * e + i] + model->exposure_background[e];
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_run_batch_submit(fpm_context* ctx, int32_t count, fpm_problem* const* problems,
                             const fpm_algorithm_params* params, fpm_result_desc* results, fpm_job** job) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    if (!job) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "job is null"));
    *job = nullptr;
    std::lock_guard<std::mutex> lock(ctx->mu);
    std::unique_ptr<fpm_job> made;
    Status st = submit_batch(ctx, count, problems, params, results, made);
    if (!st) *job = made.release();
    return finish(ctx, st);
}

int32_t fpm_spectral_run_batch_submit(fpm_context* ctx, int32_t count, const fpm_spectral_model_desc* models,
                                      const fpm_measurement_desc* measurements, const fpm_spectral_params* params,
                                      fpm_spectral_result_desc* results, fpm_job** job) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    if (!job) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "job is null"));
    *job = nullptr;
    std::lock_guard<std::mutex> lock(ctx->mu);
    std::unique_ptr<fpm_job> made;
    Status st = submit_spectral(ctx, count, models, measurements, params, results, made);
    if (!st) *job = made.release();
    return finish(ctx, st);
}

int32_t fpm_job_poll(fpm_job* job, int32_t* done) {
    if (!job || !done) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument"));
    std::lock_guard<std::mutex> lock(job->mu);
    if (!job->finished) {
        const cudaError_t q = cudaEventQuery(job->done);
        if (q == cudaErrorNotReady) {
            *done = 0;
            return FPM_OK;
        }
        if (q != cudaSuccess) {
            job->status = Status::make(FPM_ERR_CUDA, "CUDA error %s (%s)", cudaGetErrorName(q), cudaGetErrorString(q));
            job->finished = true;
        } else {
            finish_job(job);
        }
    }
    *done = 1;
    return job->status ? finish(job->ctx, job->status) : FPM_OK;
}

int32_t fpm_job_wait(fpm_job* job) {
    if (!job) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "job is null"));
    {
        std::lock_guard<std::mutex> lock(job->mu);
        if (!job->finished) {
            const cudaError_t e = cudaEventSynchronize(job->done);
            if (e != cudaSuccess) {
                job->status = Status::make(FPM_ERR_CUDA, "CUDA error %s (%s)", cudaGetErrorName(e), cudaGetErrorString(e));
                job->finished = true;
            } else {
                finish_job(job);
            }
        }
    }
    return job->status ? finish(job->ctx, job->status) : FPM_OK;
}

int32_t fpm_job_stats(fpm_job* job, fpm_run_stats* stats) {
    if (!job || !stats) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument"));
    std::lock_guard<std::mutex> lock(job->mu);
    if (!job->finished) return finish(job->ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "the job has not finished"));
    *stats = job->stats;
    return FPM_OK;
}

int32_t fpm_job_destroy(fpm_job* job) {
    if (!job) return FPM_OK;
    fpm_job_wait(job);
    delete job;
    return FPM_OK;
}

int32_t fpm_last_run_stats(const fpm_context* ctx, fpm_run_stats* stats) {
    if (!ctx || !stats) return FPM_ERR_INVALID_PARAMETER;
    *stats = ctx->stats;
    return FPM_OK;
}

}  // extern "C"

int32_t fpm_plan_create(fpm_context* ctx, int32_t count, fpm_problem* const* problems,
                        const fpm_algorithm_params* params, fpm_plan** out) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        if (!out || !params || (count > 0 && !problems))
            return Status::make(FPM_ERR_INVALID_PARAMETER, "problems, params and the output pointer must be non-null");
        FPM_CUDA(cudaSetDevice(ctx->device));
        std::unique_ptr<fpm_plan> plan;
        FPM_TRY(plan_create(ctx, count, problems, params, plan));
        *out = plan.release();
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_plan_launch(fpm_plan* plan) {
    if (!plan) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "plan is null"));
    fpm_context* ctx = plan->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        FPM_CUDA(cudaSetDevice(ctx->device));
        FPM_CUDA(cudaGraphLaunch(plan->exec, ctx->streams[0]));
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_plan_wait(fpm_plan* plan) {
    if (!plan) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "plan is null"));
    fpm_context* ctx = plan->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        FPM_CUDA(cudaSetDevice(ctx->device));
        cudaStream_t s = ctx->streams[0];
        for (auto& b : plan->buckets)
            for (fpm_problem* p : b.problems) FPM_TRY(queue_collect(p, &plan->params, nullptr, s));
        FPM_CUDA(cudaStreamSynchronize(s));
        FPM_CUDA(cudaGetLastError());
        FPM_TRY(compute_stats(plan->buckets, plan->runs, ctx->stats));
        for (auto& b : plan->buckets)
            for (fpm_problem* p : b.problems) FPM_TRY(finish_collect(p, &plan->params, nullptr));
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_plan_collect(fpm_plan* plan, fpm_result_desc* results) {
    if (!plan) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "plan is null"));
    fpm_context* ctx = plan->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        if (!results) return Status::make(FPM_ERR_INVALID_PARAMETER, "results is null");
        FPM_CUDA(cudaSetDevice(ctx->device));
        cudaStream_t s = ctx->streams[0];
        for (auto& b : plan->buckets)
            for (size_t t = 0; t < b.problems.size(); ++t)
                FPM_TRY(queue_collect(b.problems[t], &plan->params, &results[b.indices[t]], s));
        FPM_CUDA(cudaStreamSynchronize(s));
        for (auto& b : plan->buckets)
            for (size_t t = 0; t < b.problems.size(); ++t)
                FPM_TRY(finish_collect(b.problems[t], &plan->params, &results[b.indices[t]]));
        return Status::ok();
    };
    return finish(ctx, body());
}

int32_t fpm_plan_destroy(fpm_plan* plan) {
    if (!plan) return FPM_OK;
    fpm_context* ctx = plan->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    delete plan;
    return FPM_OK;
}

int32_t fpm_set_engine_grid(fpm_context* ctx, int32_t n, int32_t clusters) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    const int k = engine_grid_slot(n);
    if (k < 0) return finish(ctx, Status::make(FPM_ERR_UNSUPPORTED, "tile size %d has no frame engine", n));
    if (clusters < 0) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "clusters must be non-negative"));
    ctx->engine_grid[k] = clusters;
    return FPM_OK;
}

int32_t fpm_set_engine_ctas(fpm_context* ctx, int32_t n, int32_t ctas) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    const int k = engine_grid_slot(n);
    if (k < 0) return finish(ctx, Status::make(FPM_ERR_UNSUPPORTED, "tile size %d has no frame engine", n));
    if (ctas < 0) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "ctas must be non-negative"));
    ctx->engine_ctas[k] = ctas;
    return FPM_OK;
}

int32_t fpm_set_engine_shape(fpm_context* ctx, int32_t n, int32_t shape) {
    if (!ctx) return finish(nullptr, Status::make(FPM_ERR_INVALID_PARAMETER, "context is null"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    const int k = engine_grid_slot(n);
    if (k < 0) return finish(ctx, Status::make(FPM_ERR_UNSUPPORTED, "tile size %d has no frame engine", n));
    if (shape != FPM_ENGINE_CLUSTER && shape != FPM_ENGINE_SINGLE_CTA && shape != FPM_ENGINE_AUTO)
        return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "engine shape must be FPM_ENGINE_CLUSTER, "
                                                                   "FPM_ENGINE_SINGLE_CTA or FPM_ENGINE_AUTO"));
    if (shape != FPM_ENGINE_CLUSTER && n != 256)
        return finish(ctx, Status::make(FPM_ERR_UNSUPPORTED, "the single-CTA engine takes 256-point tiles only"));
    ctx->engine_shape[k] = shape;
    return FPM_OK;
}

int32_t fpm_engine_max_clusters(fpm_context* ctx, int32_t n, int32_t* clusters) {
    if (!ctx || !clusters) return finish(ctx, Status::make(FPM_ERR_INVALID_PARAMETER, "null argument"));
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto body = [&]() -> Status {
        FPM_CUDA(cudaSetDevice(ctx->device));
        int count = 0;
        const int k = engine_grid_slot(n);
        if (k < 0) return Status::make(FPM_ERR_UNSUPPORTED, "tile size %d has no frame engine", n);
        if (ctx->engine_shape[k] != FPM_ENGINE_CLUSTER) FPM_CUDA(fpm::engine_l2_max_active_ctas(n, &count));
        else FPM_CUDA(fpm::engine_max_active_clusters(n, &count));
        *clusters = count;
        return Status::ok();
    };
    return finish(ctx, body());
}
