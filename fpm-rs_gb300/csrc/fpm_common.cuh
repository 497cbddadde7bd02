// Shared device building blocks: complex float arithmetic, in-register DFTs
// of power-of-two length, and the twiddle table.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "twiddle256.cuh"

#define FPM_DEVICE __device__ __forceinline__

FPM_DEVICE float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FPM_DEVICE float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
FPM_DEVICE float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
FPM_DEVICE float2 cmulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
FPM_DEVICE float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
FPM_DEVICE float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
FPM_DEVICE float cnorm2(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }
FPM_DEVICE float2 cfma(float s, float2 a, float2 acc) {
    return make_float2(fmaf(s, a.x, acc.x), fmaf(s, a.y, acc.y));
}

// Multiplies by w_256^k (forward, exp(-2 pi i k/256)) or its conjugate
// (inverse). k is a compile-time constant after unrolling, so the special
// cases fold away and the general case reads the constant bank.
template <bool INV>
FPM_DEVICE float2 twiddle_const(float2 b, int k) {
    if (k == 0) return b;
    if (k == 64) return INV ? make_float2(-b.y, b.x) : make_float2(b.y, -b.x);
    if (k == 128) return make_float2(-b.x, -b.y);
    if (k == 192) return INV ? make_float2(b.y, -b.x) : make_float2(-b.y, b.x);
    float2 w = c_tw256[k];
    if (INV) w.y = -w.y;
    return cmul(b, w);
}

// Runtime-index twiddle from a shared-memory copy of the forward table.
template <bool INV>
FPM_DEVICE float2 twiddle_smem(float2 b, const float2* tw, int k) {
    float2 w = tw[k & 255];
    if (INV) w.y = -w.y;
    return cmul(b, w);
}

template <int L>
FPM_DEVICE constexpr int bit_reverse(int i) {
    int r = 0;
    for (int b = 1, m = L >> 1; b < L; b <<= 1, m >>= 1)
        if (i & b) r |= m;
    return r;
}

// One radix-2 butterfly stage of span LEN, then the next stage.
template <int L, bool INV, int LEN>
FPM_DEVICE void dft_stages(float2 (&v)[L]) {
    if constexpr (LEN <= L) {
        constexpr int HALF = LEN / 2;
        constexpr int STEP = 256 / LEN;
#pragma unroll
        for (int s = 0; s < L; s += LEN) {
#pragma unroll
            for (int j = 0; j < HALF; ++j) {
                float2 a = v[s + j];
                float2 b = twiddle_const<INV>(v[s + j + HALF], j * STEP);
                v[s + j] = cadd(a, b);
                v[s + j + HALF] = csub(a, b);
            }
        }
        dft_stages<L, INV, LEN * 2>(v);
    }
}

// In-place DFT of L values held in registers, natural order in and out:
// v[k] <- sum_n v[n] w_L^{+-nk}. Unnormalised. Radix-2 decimation in time
// with compile-time bit reversal (register renaming only).
template <int L, bool INV>
FPM_DEVICE void dft_reg(float2 (&v)[L]) {
    if constexpr (L > 1) {
#pragma unroll
        for (int i = 0; i < L; ++i) {
            const int r = bit_reverse<L>(i);
            if (r > i) {
                float2 t = v[i];
                v[i] = v[r];
                v[r] = t;
            }
        }
        dft_stages<L, INV, 2>(v);
    }
}

// A float the compiler must keep (in a register, or spilled) rather than
// recompute: values derived from FP64 kernel parameters would otherwise be
// re-derived at each use inside the pixel loops, and every conversion from
// FP64 occupies the FP64 pipe, which is narrow on GB300.
FPM_DEVICE float opaque(float x) {
    asm volatile("" : "+f"(x));
    return x;
}

// Block-wide reductions used once per frame or iteration.
FPM_DEVICE float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

FPM_DEVICE double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// 16-byte asynchronous global->shared copy that reads `src_bytes` (0, 8 or
// 16) bytes and zero-fills the rest; .cg reads through L2 only, so data
// written by other CTAs of the cluster is never served from a stale L1 line.
FPM_DEVICE void cp_async16(void* smem, const void* gmem, int src_bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}

// 8-byte asynchronous global->shared copy (through L1; read-only data).
FPM_DEVICE void cp_async8(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}

FPM_DEVICE void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Bulk prefetch of `bytes` (a multiple of 16, 16-byte aligned) into L2: one
// instruction for a whole block that a later phase reads.
FPM_DEVICE void prefetch_l2(const void* gmem, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(gmem), "r"(bytes) : "memory");
}

// Distributed shared memory: the cluster-shared address of `local` (a shared
// memory location of this CTA) in CTA `rank`, and 8-byte accesses to it.
FPM_DEVICE unsigned dsmem_address(const void* local, int rank) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(local);
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

FPM_DEVICE float2 dsmem_load(unsigned address) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(address) : "memory");
    return v;
}

FPM_DEVICE void dsmem_store(unsigned address, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};\n" ::"r"(address), "f"(v.x), "f"(v.y) : "memory");
}

// ------------------------------------------------------------ TMA staging
// A bulk tensor load completes its bytes on an mbarrier of this CTA; the
// threads wait on the phase parity, bounded in time so that a load that
// never lands cannot hang the kernel.
FPM_DEVICE unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

constexpr unsigned long long kMbarWaitNs = 2000000000ull;  // 2 s

FPM_DEVICE unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

FPM_DEVICE void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

FPM_DEVICE void mbar_inval(unsigned long long* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

FPM_DEVICE void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// True once the phase with parity `parity` has completed; false when about
// kMbarWaitNs have passed first.
FPM_DEVICE bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    unsigned long long t0 = 0;
    for (unsigned k = 0;; ++k) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((k & 255u) == 0) {
            const unsigned long long t = global_ns();
            if (k == 0) t0 = t;
            else if (t - t0 > kMbarWaitNs) return false;
        }
    }
}

// 3-D tiled bulk tensor load (box of the tensor map at coordinates x, y, z,
// innermost first) into this CTA's shared memory, completing on `bar`.
// Global data written earlier by other threads through ordinary stores is
// ordered before the load by the fence.
FPM_DEVICE void tma_load_3d(void* smem, const void* tmap, int x, int y, int z, unsigned long long* bar) {
    asm volatile("fence.proxy.async.global;\n" ::: "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(smem)),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
