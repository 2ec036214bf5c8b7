// Shared device and host helpers for the receive-chain kernels.
//
// Arithmetic discipline: every translation unit is compiled with
// --fmad=false -ftz=true, so a*b+c is a rounded multiply then a rounded add
// (never an FMA) and fp32 denormals are flushed, exactly the semantics the
// reference's twins pin (core/dsp/reference_fp.h, core/dsp/denormal_mode.h).
// Integer index, phase and recurrence arithmetic is done in the widths the
// reference's kernels use, wrapping where they wrap.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "revenant_gb300.h"

namespace rv {

// ---- host-side error plumbing (core/error.h Status -> int32 + message) ----
int32_t set_error(int32_t code, const std::string& message);
int32_t set_error_fmt(int32_t code, const char* fmt, ...);
int32_t clear_error();
int32_t cuda_status(cudaError_t err, const char* what);

inline bool is_pow2(uint64_t v) { return v != 0 && (v & (v - 1)) == 0; }

// Raises a kernel's dynamic shared memory limit on the current device to
// `bytes` when it is lower (the attribute is per device and per function).
inline int32_t ensure_shared(const void* kern, size_t bytes, const char* what) {
    cudaFuncAttributes attr;
    if (int32_t st = cuda_status(cudaFuncGetAttributes(&attr, kern), what)) return st;
    if ((size_t)attr.maxDynamicSharedSizeBytes >= bytes) return 0;
    return cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes), what);
}
inline uint32_t ilog2(uint32_t v) {
    uint32_t s = 0;
    while (s < 31 && (1u << s) < v) ++s;
    return s;
}

// ---- device helpers ----------------------------------------------------

__device__ __forceinline__ float2 ld_cf32(const rv_cf32* p) {
    return *reinterpret_cast<const float2*>(p);
}
__device__ __forceinline__ void st_cf32(rv_cf32* p, float2 v) {
    *reinterpret_cast<float2*>(p) = v;
}

// Deterministic transcendentals built only from correctly rounded + - *
// (core/dsp/vrx_reference.cpp:227-306 det_rsqrt/det_recip/det_atan2,
// core/dsp/spectrum_reference.cpp det_log2). The seeds are the reference's
// bit-trick constants and the polynomial its published coefficients, so the
// device agrees with the CPU twins bit for bit.
__device__ __forceinline__ float det_rsqrt(float value) {
    const float seed = __uint_as_float(0x5F375A86u - (__float_as_uint(value) >> 1));
    const float half_value = 0.5F * value;
    float r = seed;
#pragma unroll
    for (int i = 0; i < 4; ++i) r = r * (1.5F - half_value * (r * r));
    return r;
}

__device__ __forceinline__ float det_sqrt(float value) {
    if (!(value > 0.0F)) return 0.0F;
    return value * det_rsqrt(value);
}

__device__ __forceinline__ float det_recip(float value) {
    const float seed = __uint_as_float(0x7EF311C3u - __float_as_uint(value));
    float r = seed;
#pragma unroll
    for (int i = 0; i < 4; ++i) r = r * (2.0F - value * r);
    return r;
}

__device__ __forceinline__ float det_atan_unit(float t) {
    // (float) of the reference's double coefficients, highest order first;
    // written as double literals cast to float, as the reference writes them,
    // so the rounding path (decimal -> double -> float) is the same.
    const float u = t * t;
    float p = (float)-0.0021090222;
    p = p * u + (float)0.0122847765;
    p = p * u + (float)-0.0336503503;
    p = p * u + (float)0.0603537785;
    p = p * u + (float)-0.0853800324;
    p = p * u + (float)0.1099615976;
    p = p * u + (float)-0.1427217912;
    p = p * u + (float)0.1999923872;
    p = p * u + (float)-0.3333331929;
    p = p * u + (float)0.9999999998;
    return t * p;
}

__device__ __forceinline__ float det_atan2(float y, float x) {
    const float ay = fabsf(y);
    const float ax = fabsf(x);
    if (ay == 0.0F && ax == 0.0F) return 0.0F;
    const float numerator = (ax < ay) ? ax : ay;
    const float denominator = (ay < ax) ? ax : ay;
    const float ratio = numerator * det_recip(denominator);
    float angle = det_atan_unit(ratio);
    if (ay > ax) angle = (float)1.57079632679489661923 - angle;
    if (x < 0.0F) angle = (float)3.14159265358979323846 - angle;
    return (y < 0.0F) ? -angle : angle;
}

__device__ __forceinline__ float det_log2(float value) {
    const uint32_t bits = __float_as_uint(value);
    int exponent = (int)((bits >> 23) & 0xFFu) - 127;
    float mantissa = __uint_as_float((bits & 0x007FFFFFu) | 0x3F800000u);
    if (mantissa > 1.41421356237309505F) {
        mantissa = mantissa * 0.5F;
        exponent = exponent + 1;
    }
    const float t = (mantissa - 1.0F) * det_recip(mantissa + 1.0F);
    const float u = t * t;
    float p = 0.32059889797532520F;
    p = p * u + 0.41219858311113240F;
    p = p * u + 0.57707801635558536F;
    p = p * u + 0.96179669392597560F;
    p = p * u + 2.88539008177792681F;
    const float fraction = t * p;
    return (float)exponent + fraction;
}

// One radix-2 DIT butterfly exactly as the reference writes it
// (core/dsp/pfb_fft_reference.cpp:82-101): product b*w as mul, mul, sub /
// mul, mul, add; then the sum and the difference.
__device__ __forceinline__ void butterfly(float2& a, float2& b, float2 w) {
    const float vr = b.x * w.x - b.y * w.y;
    const float vi = b.x * w.y + b.y * w.x;
    const float2 s = make_float2(a.x + vr, a.y + vi);
    const float2 d = make_float2(a.x - vr, a.y - vi);
    a = s;
    b = d;
}

// Complex product in the reference's operand order (re = ar*br - ai*bi,
// im = ar*bi + ai*br).
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// engine::is_complex_tap (core/engine/vrx.h): modes that hand out baseband.
__host__ __device__ __forceinline__ bool is_complex_demod(uint32_t m) {
    return m == RV_DEMOD_RAW || m == RV_DEMOD_P25P1 || m == RV_DEMOD_DSTAR || m == RV_DEMOD_TETRA ||
           m == RV_DEMOD_DMR;
}

__device__ __forceinline__ uint32_t brev(uint32_t v, uint32_t stages) {
    return stages == 0 ? 0u : (__brev(v) >> (32u - stages));
}

__device__ __forceinline__ int32_t sext16(uint32_t raw) { return ((int32_t)(raw << 16)) >> 16; }

// One raw sample at ring position pos (cs16: one 32-bit word per sample,
// cu8: two per word), converted exactly as the plain convert kernel converts
// it (core/dsp/convert.h: int16 * 2^-15; (code - 127.5) * 0x3C008081).
template <int FMT>
__device__ __forceinline__ float2 convert_raw(const uint32_t* __restrict__ raw, uint32_t pos) {
    if (FMT == RV_FORMAT_CS16) {
        const uint32_t w = __ldg(&raw[pos]);
        return make_float2((float)sext16(w & 0xFFFFu) * 0.000030517578125F,
                           (float)sext16(w >> 16) * 0.000030517578125F);
    } else {  // RV_FORMAT_CU8
        const uint32_t w = __ldg(&raw[pos >> 1]);
        const int shift = (int)((pos & 1u) << 4);
        const uint32_t i_raw = (w >> shift) & 0xFFu;
        const uint32_t q_raw = (w >> (shift + 8)) & 0xFFu;
        return make_float2(((float)i_raw - 127.5F) * 0.00784313772F,
                           ((float)q_raw - 127.5F) * 0.00784313772F);
    }
}

}  // namespace rv
