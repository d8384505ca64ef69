// Shared device/host helpers for the strands-to-cards raster kernels (sm_103a).
//
// Exactness: every translation unit is compiled with --fmad=false, so a multiply-add
// is fused only where it is written as fmaf().  The fused sites below are the ones the
// reference's nvcc build fuses (established by running the reference's own kernels on
// the same inputs); with them, pixel coverage, spans, t1/z and barycentrics come out
// bit-identical to the reference.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "s2c.h"

namespace s2c {

constexpr int kMaxDevices = 64;   // per-device launch caches (device index mod 64)

// ---- status / errors -------------------------------------------------------------
void set_error(const char* fmt, ...);
s2c_status cuda_status(cudaError_t e, const char* what);
#define S2C_CHECK_LAUNCH(what)                                              \
    do {                                                                    \
        cudaError_t e__ = cudaGetLastError();                               \
        if (e__ != cudaSuccess) return ::s2c::cuda_status(e__, what);       \
    } while (0)
#define S2C_REQUIRE(cond, ...)                                              \
    do {                                                                    \
        if (!(cond)) { ::s2c::set_error(__VA_ARGS__); return S2C_ERR_INVALID; } \
    } while (0)

// the calling thread's current device, as an index into the per-device caches below
inline int current_device_slot() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev & (kMaxDevices - 1);
}

// SM count of the current device (cached per device)
inline int num_sms() {
    static std::atomic<int> cache[kMaxDevices];
    const int slot = current_device_slot();
    int n = cache[slot].load(std::memory_order_relaxed);
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 152;
        cache[slot].store(n, std::memory_order_relaxed);
    }
    return n;
}

inline unsigned grid_for(int64_t n, int threads, int64_t cap = 1 << 30) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// n / d for 0 <= n < 2^31 by multiply-high (Granlund & Montgomery, "Division by invariant
// integers using multiplication", 1994): l = ceil(log2 d), m = 2^32 (2^l - d) / d + 1,
// q = (mulhi(m, n) + n) >> l.
struct FastDiv {
    uint32_t d = 1, m = 0, l = 0;
    FastDiv() = default;
    explicit FastDiv(uint32_t dv) : d(dv ? dv : 1) {
        l = 0;
        while ((1ull << l) < d) ++l;
        m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(m, n) + n) >> l; }
};

// carve aligned sub-buffers out of a caller workspace
struct Carver {
    char* base;
    size_t cap, off = 0;
    Carver(void* b, size_t c) : base((char*)b), cap(c) {}
    template <class T> T* take(size_t n) {
        off = align_up(off, 256);
        T* p = (T*)(base + off);
        off += n * sizeof(T);
        return p;
    }
    bool ok() const { return off <= cap; }
};

// ---- exact FP32 arithmetic -----------------------------------------------------------
// float -> int: cvt.rzi.s32.f32 (truncation, saturating, NaN -> 0), as the reference's
// static_cast<int>() compiles to.
__device__ __forceinline__ int f2i(float f) { return __float2int_rz(f); }
__device__ __forceinline__ float fmax_macro(float a, float b) { return a > b ? a : b; }

// One DDA primitive (dda.cu:9-87): major axis, slope, clamped start and the sweep offsets.
struct Span {
    float sx, sy, slope, off0, off1;
    float axis;     // 0: x-major sweep, 1: y-major sweep
    int count;      // fragments before bounds / depth rejection
};

// Pixel-space endpoint (dda.cu:25-36); Unit: w == 1, where the division is exact and skipped
template <bool Unit>
__device__ __forceinline__ void dda_pixel(float4 p, float fW, float fH, float& x, float& y) {
    const float xn = Unit ? p.x : __fdiv_rn(p.x, p.w);
    const float yn = Unit ? p.y : __fdiv_rn(p.y, p.w);
    x = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(xn, 1.f)), fW);
    y = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(1.f, yn)), fH);
}

template <bool Unit>
__device__ __forceinline__ Span dda_span_t(float4 p0, float4 p1, int H, int W) {
    Span s;
    const float fH = (float)H, fW = (float)W;
    float x0, y0, x1, y1;
    dda_pixel<Unit>(p0, fW, fH, x0, y0);
    dda_pixel<Unit>(p1, fW, fH, x1, y1);
    const float dx = __fsub_rn(x1, x0), dy = __fsub_rn(y1, y0);
    s.sx = s.sy = s.slope = s.off0 = s.off1 = 0.f;
    s.axis = 0.f;
    s.count = 0;
    if (dx == 0.f && dy == 0.f) return s;
    if (fabsf(dx) >= fabsf(dy)) {
        const float sl = __fdiv_rn(dy, dx);
        if (x0 > x1) { float t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; }
        const float fsx = fmax_macro(floorf(x0), 0.f);
        s.sx = fsx;
        s.sy = __fmaf_rn(sl, __fsub_rn(fsx, x0), y0);
        s.slope = sl;
        s.off0 = __fsub_rn(x0, fsx);
        s.off1 = __fsub_rn(x1, fsx);
        s.axis = 0.f;
        const int xs = f2i(fsx);
        const int xe = min(f2i(floorf(x1)), W - 1) + 1;
        const int c = (int)((unsigned)xe - (unsigned)xs);
        s.count = c > 0 ? c : 0;
    } else {
        const float sl = __fdiv_rn(dx, dy);
        if (y0 > y1) { float t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; }
        const float fsy = fmax_macro(floorf(y0), 0.f);
        s.sy = fsy;
        s.sx = __fmaf_rn(sl, __fsub_rn(fsy, y0), x0);
        s.slope = sl;
        s.off0 = __fsub_rn(y0, fsy);
        s.off1 = __fsub_rn(y1, fsy);
        s.axis = 1.f;
        const int ys = f2i(fsy);
        const int ye = min(f2i(floorf(y1)), H - 1) + 1;
        const int c = (int)((unsigned)ye - (unsigned)ys);
        s.count = c > 0 ? c : 0;
    }
    return s;
}

// Orthographic views (w = 1 at both ends) take a copy without the four divisions; a real
// branch, so the divisions are not evaluated and discarded.
__device__ __forceinline__ Span dda_span(float4 p0, float4 p1, int H, int W) {
    if (p0.w == 1.0f && p1.w == 1.0f) return dda_span_t<true>(p0, p1, H, W);
    return dda_span_t<false>(p0, p1, H, W);
}

// Sample point of fragment k (dda.cu:185-193); the minor coordinate is not fused.
__device__ __forceinline__ void dda_sample(const Span& s, int k, float& x, float& y) {
    const float d = fminf(fmaxf(__fadd_rn((float)k, 0.5f), s.off0), s.off1);
    if (s.axis == 0.f) {
        x = __fadd_rn(s.sx, d);
        y = __fadd_rn(s.sy, __fmul_rn(d, s.slope));
    } else {
        x = __fadd_rn(s.sx, __fmul_rn(d, s.slope));
        y = __fadd_rn(s.sy, d);
    }
}

// Perspective-correct t1 (dda.cu:124-144)
__device__ __forceinline__ float dda_t1(float4 p0, float4 p1, float x, float y, float axis, int H, int W) {
    float a, b;
    if (axis == 0.f) {
        const float q = __fadd_rn(-1.f, __fmul_rn(2.f, __fdiv_rn(x, (float)W)));
        a = __fmaf_rn(-q, p0.w, p0.x);
        b = __fmaf_rn(-q, p1.w, p1.x);
    } else {
        const float q = __fadd_rn(-1.f, __fmul_rn(2.f, __fdiv_rn(y, (float)H)));
        a = __fmaf_rn(-q, p0.w, -p0.y);
        b = __fmaf_rn(-q, p1.w, -p1.y);
    }
    const float t0 = fabsf(b), t1 = fabsf(a);
    const float den = __fadd_rn(t0, t1);
    if (den < 1e-6f) return 0.5f;
    return __fdiv_rn(t1, den);
}

// Depth of the sample (dda.cu:211-214): t0*a + t1*b is fused on its second product.
__device__ __forceinline__ float dda_z(float4 p0, float4 p1, float t1) {
    const float t0 = __fsub_rn(1.f, t1);
    const float pz = __fmaf_rn(t1, p1.z, __fmul_rn(t0, p0.z));
    const float pw = __fmaf_rn(t1, p1.w, __fmul_rn(t0, p0.w));
    return __fdiv_rn(pz, pw);
}

__device__ __forceinline__ bool z_ok(float z) { return isfinite(z) && z >= -1.f && z <= 1.f; }

// Depth test skipped when both ends are finite, 1e-30 <= w <= 1e30 and |z| <= 0.999 w:
// then for every t1 in [0, 1] the reference's z = (t0 z0 + t1 z1) / (t0 w0 + t1 w1),
// rounded, has |z| <= 0.999 (1 + 5 eps) < 1, so every fragment passes.
__device__ __forceinline__ bool depth_always_passes(float4 a, float4 b) {
    auto ok = [](float4 p) {
        return isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && p.w >= 1e-30f && p.w <= 1e30f &&
               fabsf(p.z) <= 0.999f * p.w;
    };
    return ok(a) && ok(b);
}


// The reference carries the primitive id as float(e + 1) and casts it back.
__device__ __forceinline__ int prim_roundtrip(int e) { return f2i((float)(e + 1)) - 1; }

}  // namespace s2c
