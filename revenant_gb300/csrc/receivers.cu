// Batched receivers: every virtual receiver of the chain in one launch per
// stage, over a work list of (receiver, output run) items.
//
// The arithmetic per output is the reference's (vrx_fine.comp:270-369,
// vrx_demod.comp:445-659; twins core/dsp/vrx_reference.cpp:489-917), so every
// fine sample and audio frame is bit-identical to the plain per-receiver
// kernels. Three redundancies of the per-receiver dispatch are removed without
// changing a rounding:
//
//  * Pre-blended polyphase taps. A receiver's (phase, blend) pair depends only
//    on frac(j) = j * (Fc mod Fd) mod Fd for fine output j, which repeats with
//    period Fd / gcd(Fc mod Fd, Fd) (48 outputs for a 625 kS/s channel
//    resampled to 48 kS/s, 336 for 336 kS/s). The blended taps
//    g0 * (1 - b) + g1 * b are computed once per pattern phase, with the same
//    two multiplies and one add, and the per-output FIR reads them: half the
//    tap-table reads and six fewer flops per tap.
//  * The detector once per fine sample. The reference evaluates the FM
//    discriminator, the AM magnitude and its DC-removal FIR inside the audio
//    FIR's tap loop, i.e. audio_taps (x dc_taps for AM) times per audio frame.
//    Here the detector runs once per fine sample into a ring and the audio FIR
//    reads it: identical values, since the detector is a pure function of the
//    fine samples.
//  * One launch per stage for all receivers, each CTA staging the input window
//    of its run in shared memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include "carrier.cuh"
#include "common.cuh"
#include "receivers.cuh"

namespace rv {
namespace {

__global__ void k_lerp_table(const rv_cf32* __restrict__ taps, float2* __restrict__ out, uint32_t T, uint32_t P,
                             uint32_t period, uint32_t step_rem, uint32_t fd, float inv_fd) {
    const uint32_t total = period * T;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const uint32_t pp = idx / T, k = idx % T;
        // frac of any fine output j with j mod period == pp
        const uint32_t frac = (uint32_t)(((uint64_t)pp * step_rem) % fd);
        const uint32_t scaled = frac * P;
        const uint32_t phase = scaled / fd;
        const uint32_t blend_num = scaled - phase * fd;
        const float blend = (float)blend_num * inv_fd;
        const float blend_c = 1.0F - blend;
        const uint32_t slot = phase + k * P;
        const float2 g0 = ld_cf32(&taps[slot]);
        const float2 g1 = ld_cf32(&taps[slot + 1u]);
        // tap-major: the 32 lanes of a warp hold 32 consecutive outputs, i.e.
        // consecutive pattern phases, so tap k of all of them is contiguous
        out[(uint64_t)k * period + pp] = make_float2(g0.x * blend_c + g1.x * blend, g0.y * blend_c + g1.y * blend);
    }
}

// ---- fine stage ---------------------------------------------------------

// Next item index from the launch's queue (one atomic per CTA per item).
__device__ __forceinline__ uint32_t next_item(uint32_t* queue, uint32_t* slot) {
    __syncthreads();
    if (threadIdx.x == 0) *slot = atomicAdd(queue, 1u);
    __syncthreads();
    return *slot;
}

// Item `it` of a span list: the receiver by binary search over the prefix
// sums (the largest r with prefix[r] <= it is the one that owns it; empty
// receivers share their prefix with the next), then the item's range.
__device__ __forceinline__ WorkItem span_item(const SpanList& sl, const RxDev* __restrict__ rxs, uint32_t it) {
    uint32_t lo = 0, hi = sl.nrx;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (sl.prefix[mid] <= it) lo = mid;
        else hi = mid;
    }
    const RxRun run = sl.runs[lo];
    const uint32_t k = it - sl.prefix[lo];
    WorkItem w{};
    w.rx = lo;
    if (sl.audio == 0) {
        const uint32_t size = rxs[lo].det_item;
        w.first = run.det_first + (uint64_t)k * size;
        w.count = min(size, run.det_count - k * size);
    } else {
        const uint32_t size = rxs[lo].audio_item;
        w.first = run.audio_first + (uint64_t)k * size;
        w.count = min(size, run.audio_count - k * size);
        w.out = run.audio_out + (uint64_t)k * size * rxs[lo].channels;
    }
    return w;
}

__global__ void __launch_bounds__(kRxThreads)
k_fine_batched(const RxDev* __restrict__ rxs, const WorkItem* __restrict__ items, uint32_t nitems,
               const float2* __restrict__ chan, uint32_t window_cap, uint32_t* queue, const uint32_t* dyn) {
    extern __shared__ float2 xs[];
    __shared__ uint32_t s_it;
    __shared__ RxDev rx;
    if (dyn != nullptr) nitems = *dyn;
    for (uint32_t it = next_item(queue, &s_it); it < nitems; it = next_item(queue, &s_it)) {
        const WorkItem item = items[it];
        if (threadIdx.x == 0) rx = rxs[item.rx];
        __syncthreads();
        const uint32_t T = rx.taps;
        const uint64_t base = item.n0 - (T - 1u);
        const uint32_t len = item.window < window_cap ? item.window : window_cap;
        for (uint32_t e = threadIdx.x; e < len; e += blockDim.x)
            xs[e] = chan[(uint64_t)rx.chan_base + (uint32_t)((base + e) & rx.chan_mask)];
        __syncthreads();
        const uint32_t s_frac0 = item.frac0, s_p0 = item.p0;
        const uint32_t i = threadIdx.x;
        const uint32_t fd = rx.out_rate;
        const uint32_t acc = s_frac0 + i * rx.step_rem;
        const uint32_t carry = acc / fd;
        const uint32_t n_rel = i * rx.step_whole + carry;
        // n_rel + T - 1 < len always holds for items the chain builds; the
        // guard keeps every shared-memory read inside the staged window
        if (i < item.count && n_rel + T - 1u < len) {
            const float2* w = xs + n_rel + T - 1u;  // w[-k] = x[n(j) - k]
            float ar = 0.0F, ai = 0.0F;
            if (rx.lerped != nullptr) {
                const uint32_t pp = (s_p0 + i) % rx.period;
                const uint32_t stride = rx.period;
                const float2* __restrict__ tp = rx.lerped + pp;
#pragma unroll 4
                for (uint32_t k = 0; k < T; ++k) {
                    const float2 s = w[-(int)k];
                    const float2 t = __ldg(&tp[(uint64_t)k * stride]);
                    ar = ar + (s.x * t.x - s.y * t.y);
                    ai = ai + (s.x * t.y + s.y * t.x);
                }
            } else {
                // blend on the fly, exactly as the plain kernel does
                const uint32_t frac = acc - carry * fd;
                const uint32_t scaled = frac * rx.phases;
                const uint32_t phase = scaled / fd;
                const uint32_t blend_num = scaled - phase * fd;
                const float blend = (float)blend_num * rx.inv_out_rate;
                const float blend_c = 1.0F - blend;
                for (uint32_t k = 0; k < T; ++k) {
                    const uint32_t slot = phase + k * rx.phases;
                    const float2 g0 = rx.taps_raw[slot];
                    const float2 g1 = rx.taps_raw[slot + 1u];
                    const float tr = g0.x * blend_c + g1.x * blend;
                    const float ti = g0.y * blend_c + g1.y * blend;
                    const float2 s = w[-(int)k];
                    ar = ar + (s.x * tr - s.y * ti);
                    ai = ai + (s.x * ti + s.y * tr);
                }
            }
            const uint64_t j = item.first + i;
            const uint64_t phi = rx.nco_delta * j;
            const uint32_t idx = (rx.nco_log2 == 0) ? 0u : ((uint32_t)(phi >> 32) >> (32u - rx.nco_log2));
            const float2 rot = rx.nco[idx];
            rx.fine[(uint32_t)j & rx.fine_mask] = make_float2(ar * rot.x - ai * rot.y, ar * rot.y + ai * rot.x);
        }
        __syncthreads();
    }
}

// ---- fine stage, tap table resident in shared memory ----------------------
//
// One CTA per unit: the receiver's blended taps ([T][period], tap-major) are
// copied into shared memory once, then each item of the unit stages its input
// window after the table and every thread computes one fine output with both
// operands in shared memory (consecutive lanes read consecutive pattern phases
// of one tap row: no bank conflicts on the taps).

__global__ void __launch_bounds__(kUnitThreads)
k_fine_units(const RxDev* __restrict__ rxs, const WorkItem* __restrict__ items, const FineUnit* __restrict__ units,
             uint32_t nunits, const float2* __restrict__ chan, uint32_t shared_float2s, uint32_t* queue,
             const uint32_t* dyn) {
    extern __shared__ float2 sm[];
    __shared__ uint32_t s_it;
    __shared__ RxDev rx;
    if (dyn != nullptr) nunits = *dyn;
    for (uint32_t u = next_item(queue, &s_it); u < nunits; u = next_item(queue, &s_it)) {
        const FineUnit unit = units[u];
        if (threadIdx.x == 0) rx = rxs[unit.rx];
        __syncthreads();
        const uint32_t T = rx.taps, period = rx.period;
        const uint32_t rows = unit.rows < T ? unit.rows : T;
        const bool resident = rows == T;
        const uint32_t chunk = rows * period;  // float2 of table in shared memory
        if (resident)
            for (uint32_t e = threadIdx.x; e < chunk; e += blockDim.x) sm[e] = __ldg(&rx.lerped[e]);
        float2* xs = sm + chunk;
        const uint32_t cap = shared_float2s - chunk;
        for (uint32_t k = 0; k < unit.items; ++k) {
            const WorkItem item = items[unit.first_item + k];
            const uint64_t base = item.n0 - (T - 1u);
            const uint32_t len = item.window < cap ? item.window : cap;
            __syncthreads();  // the previous item's readers are done with xs
            for (uint32_t e = threadIdx.x; e < len; e += blockDim.x)
                xs[e] = chan[(uint64_t)rx.chan_base + (uint32_t)((base + e) & rx.chan_mask)];
            const uint32_t i = threadIdx.x;
            const uint32_t fd = rx.out_rate;
            const uint32_t acc = item.frac0 + i * rx.step_rem;
            const uint32_t carry = acc / fd;
            const uint32_t n_rel = i * rx.step_whole + carry;
            const bool active = i < item.count && n_rel + T - 1u < len;
            const float2* w = xs + n_rel + T - 1u;  // w[-q] = x[n(j) - q]
            const uint32_t pp = active ? (item.p0 + i) % period : 0u;
            float ar = 0.0F, ai = 0.0F;
            for (uint32_t q0 = 0; q0 < T; q0 += rows) {
                const uint32_t q1 = (q0 + rows < T) ? q0 + rows : T;
                if (!resident) {
                    __syncthreads();  // everyone is done with the previous chunk
                    const float2* src = rx.lerped + (uint64_t)q0 * period;
                    const uint32_t n = (q1 - q0) * period;
                    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) sm[e] = __ldg(&src[e]);
                }
                __syncthreads();  // window (and chunk) staged
                if (active) {
                    const float2* tp = sm + pp;
#pragma unroll 4
                    for (uint32_t q = q0; q < q1; ++q) {
                        const float2 sv = w[-(int)q];
                        const float2 t = tp[(q - q0) * period];
                        ar = ar + (sv.x * t.x - sv.y * t.y);
                        ai = ai + (sv.x * t.y + sv.y * t.x);
                    }
                }
            }
            if (active) {
                const uint64_t j = item.first + i;
                const uint64_t phi = rx.nco_delta * j;
                const uint32_t idx = (rx.nco_log2 == 0) ? 0u : ((uint32_t)(phi >> 32) >> (32u - rx.nco_log2));
                const float2 rot = rx.nco[idx];
                rx.fine[(uint32_t)j & rx.fine_mask] = make_float2(ar * rot.x - ai * rot.y, ar * rot.y + ai * rot.x);
            }
        }
    }
}

// ---- carrier loop (SAM / DSB): serial per receiver ----------------------

__global__ void k_carrier_batched(const RxDev* __restrict__ rxs, const WorkItem* __restrict__ items, uint32_t nitems,
                                  const uint32_t* dyn) {
    const uint32_t it = blockIdx.x * blockDim.x + threadIdx.x;
    if (dyn != nullptr) nitems = *dyn;
    if (it >= nitems) return;
    const WorkItem item = items[it];
    const RxDev& rx = rxs[item.rx];
    rv_vrx_carrier_params p = rx.carrier;
    p.in_mask = rx.fine_mask;
    p.in_offset = (uint32_t)item.first & rx.fine_mask;
    p.count = item.count;
    p.flags = (uint32_t)item.out;  // the reset flag travels in `out`
    p.shift = 0.0F;
    carrier_loop(reinterpret_cast<const rv_cf32*>(rx.nco), reinterpret_cast<rv_cf32*>(rx.fine), rx.carrier_state,
                 rx.carrier_power, rx.nco_log2, p);
}

// ---- detector, once per fine sample ---------------------------------------

// acc = (acc.lo + lo, acc.hi + hi), two rounded adds in one instruction
__device__ __forceinline__ void add_pair(uint64_t& acc, float lo, float hi) {
    asm("{\n .reg .b64 t;\n mov.b64 t, {%1, %2};\n add.rn.ftz.f32x2 %0, %0, t;\n}\n" : "+l"(acc) : "f"(lo), "f"(hi));
}
__device__ __forceinline__ void unpack_pair(uint64_t acc, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc));
}
// fast mode: acc = (acc.lo + lo * w, acc.hi + hi * w), one fused packed
// multiply-add (each lane rounded once)
__device__ __forceinline__ void fma_pair(uint64_t& acc, float lo, float hi, float w) {
    asm("{\n .reg .b64 x, y;\n mov.b64 x, {%1, %2};\n mov.b64 y, {%3, %3};\n fma.rn.ftz.f32x2 %0, x, y, %0;\n}\n"
        : "+l"(acc)
        : "f"(lo), "f"(hi), "f"(w));
}

// FAST (the chain's fast mode): the DC-removal FIR's products and sums as
// fused multiply-adds, to a stated tolerance rather than the reference's bits.
template <bool FAST>
__global__ void __launch_bounds__(kRxThreads)
k_detect_batched(const RxDev* __restrict__ rxs, SpanList spans, uint32_t nitems, uint32_t window_cap, uint32_t* queue,
                 const uint32_t* dyn) {
    extern __shared__ __align__(16) float sd[];
    __shared__ uint32_t s_it;
    __shared__ RxDev rx;
    __shared__ WorkItem s_item;
    if (dyn != nullptr) nitems = *dyn;
    for (uint32_t it = next_item(queue, &s_it); it < nitems; it = next_item(queue, &s_it)) {
        if (threadIdx.x == 0) {
            s_item = span_item(spans, rxs, it);
            rx = rxs[s_item.rx];
        }
        __syncthreads();
        const WorkItem item = s_item;
        const uint32_t mode = rx.mode;
        const uint32_t i = threadIdx.x;
        const uint32_t first = (uint32_t)item.first;  // ring arithmetic is modulo the mask
        if (mode == RV_DEMOD_AM || mode == RV_DEMOD_SAM) {
            // DC removal FIR over |z| (AM) or Re z (SAM), four consecutive
            // outputs per thread: each staged input and each weight is read
            // once per four multiply-adds; every output still sums its terms
            // in ascending weight order, one rounded multiply and one rounded
            // add each, as the reference's detect() does.
            const uint32_t dc = rx.dc_taps;
            float* dws = sd + window_cap;  // weights, after the window (16-byte aligned)
            // Stage the inputs at an offset o in [4, 8) chosen so that the
            // window base v of every thread is 16-byte aligned and the last
            // group's look-ahead read stays inside the allocation.
            const uint32_t o = 4u + ((4u - ((dc - 1u) & 3u)) & 3u);
            const uint32_t len = item.count + dc - 1u + 3u;  // +3: the last thread's tail
            const uint32_t start = first - (dc - 1u);
            for (uint32_t e = threadIdx.x; e < len && o + e < window_cap; e += blockDim.x) {
                const float2 z = rx.fine[(start + e) & rx.fine_mask];
                sd[o + e] = (mode == RV_DEMOD_AM) ? det_sqrt(z.x * z.x + z.y * z.y) : z.x;
            }
            for (uint32_t e = threadIdx.x; e < dc; e += blockDim.x) dws[e] = rx.weights[rx.audio_taps + e];
            __syncthreads();
            const uint32_t i0 = 4u * i;
            if (i0 < item.count && o + i0 + 3u + dc - 1u < (o + len < window_cap ? o + len : window_cap)) {
                const float* v = sd + o + i0 + dc - 1u;  // v[r - w] = input at fine (first + i0 + r - w)
                // x_r holds v[r - w] at the top of each group of four steps:
                //   step w  : a_r += v[r-w]   * wt[w]    -> x0 x1 x2 x3
                //   step w+1: a_r += v[r-w-1] * wt[w+1]  -> y  x0 x1 x2
                //   step w+2: a_r += v[r-w-2] * wt[w+2]  -> z  y  x0 x1
                //   step w+3: a_r += v[r-w-3] * wt[w+3]  -> u  z  y  x0
                // with (n, u, z, y) = v[-w-4 .. -w-1], one aligned 16-byte load,
                // and the next group's x0..x3 = n, u, z, y.
                // a01 = (a0, a1) and a23 = (a2, a3) are packed pairs: each step
                // makes its four products with rounded scalar multiplies and
                // adds them with two rounded packed adds (add.rn.ftz.f32x2,
                // lane for lane the scalar add), so every output keeps its bits
                uint64_t a01 = 0, a23 = 0;
                const float4 first4 = *reinterpret_cast<const float4*>(v);
                float x0 = first4.x, x1 = first4.y, x2 = first4.z, x3 = first4.w;
                uint32_t w = 0;
                // unrolled four groups deep: the window's rotation is then a
                // renaming of registers rather than moves
#pragma unroll 4
                for (; w + 4u <= dc; w += 4u) {
                    const float4 nz = *reinterpret_cast<const float4*>(v - (int)w - 4);
                    const float4 wt = *reinterpret_cast<const float4*>(dws + w);
                    const float y = nz.w, z = nz.z, u = nz.y;
                    if (FAST) {
                        fma_pair(a01, x0, x1, wt.x); fma_pair(a23, x2, x3, wt.x);
                        fma_pair(a01, y, x0, wt.y); fma_pair(a23, x1, x2, wt.y);
                        fma_pair(a01, z, y, wt.z); fma_pair(a23, x0, x1, wt.z);
                        fma_pair(a01, u, z, wt.w); fma_pair(a23, y, x0, wt.w);
                    } else {
                        add_pair(a01, x0 * wt.x, x1 * wt.x); add_pair(a23, x2 * wt.x, x3 * wt.x);
                        add_pair(a01, y * wt.y, x0 * wt.y); add_pair(a23, x1 * wt.y, x2 * wt.y);
                        add_pair(a01, z * wt.z, y * wt.z); add_pair(a23, x0 * wt.z, x1 * wt.z);
                        add_pair(a01, u * wt.w, z * wt.w); add_pair(a23, y * wt.w, x0 * wt.w);
                    }
                    x3 = y;
                    x2 = z;
                    x1 = u;
                    x0 = nz.x;
                }
                float a0, a1, a2, a3;
                unpack_pair(a01, a0, a1);
                unpack_pair(a23, a2, a3);
                for (; w < dc; ++w) {
                    const float wt = dws[w];
                    a0 = a0 + x0 * wt; a1 = a1 + x1 * wt; a2 = a2 + x2 * wt; a3 = a3 + x3 * wt;
                    x3 = x2;
                    x2 = x1;
                    x1 = x0;
                    x0 = v[-(int)w - 1];
                }
                const float acc[4] = {a0, a1, a2, a3};
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (i0 + (uint32_t)r < item.count) rx.det[(first + i0 + (uint32_t)r) & rx.fine_mask] = v[r] - acc[r];
            }
        } else {
            // one detector value per fine sample, items of up to four per thread
            for (uint32_t k = i; k < item.count; k += blockDim.x) {
                const uint32_t f = first + k;
                const float2 z = rx.fine[f & rx.fine_mask];
                float d;
                if (mode == RV_DEMOD_NFM || mode == RV_DEMOD_WFM) {
                    const float2 q = rx.fine[(f - 1u) & rx.fine_mask];
                    const float pr = z.x * q.x + z.y * q.y;
                    const float pi = z.y * q.x - z.x * q.y;
                    d = det_atan2(pi, pr);
                } else {
                    d = z.x;
                }
                rx.det[f & rx.fine_mask] = d;
            }
        }
        __syncthreads();
    }
}

// ---- audio FIR with decimation, mono or stereo ----------------------------

// FAST (the chain's fast mode): the mono FIR's products and sums as fused
// multiply-adds.
template <bool FAST>
__global__ void __launch_bounds__(kRxThreads)
k_audio_batched(const RxDev* __restrict__ rxs, SpanList spans, uint32_t nitems, float* __restrict__ audio,
                uint32_t window_cap, uint32_t weights_cap, uint32_t* queue, const uint32_t* dyn) {
    extern __shared__ __align__(16) float sd[];
    __shared__ uint32_t s_it;
    __shared__ RxDev rx;
    __shared__ WorkItem s_item;
    if (dyn != nullptr) nitems = *dyn;
    for (uint32_t it = next_item(queue, &s_it); it < nitems; it = next_item(queue, &s_it)) {
        if (threadIdx.x == 0) {
            s_item = span_item(spans, rxs, it);
            rx = rxs[s_item.rx];
        }
        __syncthreads();
        const WorkItem item = s_item;
        const uint32_t i = threadIdx.x;
        const uint32_t dec = rx.decimation;
        const uint32_t first_index = (uint32_t)(item.first * dec);  // fine index of the first frame, mod 2^32
        float* out = audio + item.out;
        if (is_complex_demod(rx.mode)) {
            if (i < item.count) {
                const float2 z = rx.fine[(first_index + i * dec) & rx.fine_mask];
                out[2u * i] = z.x * rx.gain;
                out[2u * i + 1u] = z.y * rx.gain;
            }
            __syncthreads();
            continue;
        }
        // detector window [first_index - reach, last index], then the weights
        const uint32_t len = (item.count - 1u) * dec + rx.reach + 1u;
        const uint32_t start = first_index - rx.reach;
        for (uint32_t e = threadIdx.x; e < len && e < window_cap; e += blockDim.x)
            sd[e] = rx.det[(start + e) & rx.fine_mask];
        float* ws = sd + window_cap;
        if (rx.channels == 2u) {
            // packed: {w[t], rotation[2t], rotation[2t + 1], 0} per tap, then the pilot pairs
            const uint32_t Ta = rx.audio_taps, pilot_base = Ta + rx.dc_taps;
            const uint32_t rotation_base = pilot_base + 2u * rx.pilot_taps;
            const uint32_t nw = stereo_weight_floats(Ta, rx.pilot_taps);
            for (uint32_t e = threadIdx.x; e < nw && e < weights_cap; e += blockDim.x) {
                float v;
                if (e < 4u * Ta) {
                    const uint32_t t = e >> 2, c = e & 3u;
                    v = c == 0u ? rx.weights[t] : c == 3u ? 0.0F : rx.weights[rotation_base + 2u * t + (c - 1u)];
                } else {
                    v = rx.weights[pilot_base + (e - 4u * Ta)];
                }
                ws[e] = v;
            }
        } else {
            // the taps, then the four shifted copies (mono_weight_floats)
            const uint32_t Ta = rx.audio_taps, C0 = mono_copy_base(Ta), S = mono_copy_stride(Ta);
            const uint32_t nw = mono_weight_floats(Ta);
            for (uint32_t e = threadIdx.x; e < nw && e < weights_cap; e += blockDim.x) {
                float v = 0.0F;
                if (e < Ta) {
                    v = rx.weights[e];
                } else if (e >= C0) {
                    const uint32_t h = (e - C0) / S + 1u, jj = (e - C0) % S;
                    if (jj + h < Ta) v = rx.weights[jj + h];
                }
                ws[e] = v;
            }
        }
        __syncthreads();
        if (i < item.count && rx.reach + i * dec < (len < window_cap ? len : window_cap)) {
            const float* v = sd + rx.reach + i * dec;  // v[-t] = detector at (index - t)
            const float* w = ws;
            if (rx.channels == 2u) {
                const float4* wq = reinterpret_cast<const float4*>(w);
                const float2* wp = reinterpret_cast<const float2*>(w + 4u * rx.audio_taps);
                const float* pv = v - (int)(rx.audio_taps / 2u);
                uint64_t pacc = 0;  // (pr, pi), added as one packed pair
                for (uint32_t k = 0; k < rx.pilot_taps; ++k) {
                    const float comp = pv[-(int)k];
                    const float2 pw = wp[k];
                    add_pair(pacc, comp * pw.x, comp * pw.y);
                }
                float pr, pi;
                unpack_pair(pacc, pr, pi);
                const float sr = pr * rx.gain, si = pi * rx.gain;
                const float rr = sr * sr, ii = si * si;
                const float power = rr + ii;
                const float inverse = det_recip((power < 2.0e-5F) ? 2.0e-5F : power);
                const float cross = sr * si;
                const float cos_two = (ii - rr) * inverse;
                const float sin_two = (-2.0F * cross) * inverse;
                const float locked = (power >= 2.0e-5F) ? 1.0F : 0.0F;
                uint64_t sd_acc = 0;  // (sum, diff), added as one packed pair
                for (uint32_t t = 0; t < rx.audio_taps; ++t) {
                    const float4 q = wq[t];
                    const float weighted = v[-(int)t] * q.x;
                    const float ref = sin_two * q.y - cos_two * q.z;
                    add_pair(sd_acc, weighted, weighted * ref);
                }
                float sum, diff;
                unpack_pair(sd_acc, sum, diff);
                const float gated = diff * locked;
                out[2u * i] = (sum + gated) * rx.gain;
                out[2u * i + 1u] = (sum - gated) * rx.gain;
            } else {
                // taps 0..h-1 from the frame's first quad of samples, then
                // aligned four-tap steps (samples as 16-byte vectors read
                // backwards, weights from the copy shifted by h), then the
                // rest; every product is rounded and added in tap order
                const uint32_t Ta = rx.audio_taps;
                const uint32_t base = rx.reach + i * dec;  // v = sd + base
                const uint32_t q0 = base & ~3u;
                const uint32_t h = base - q0 + 1u;
                const uint32_t hp = h < Ta ? h : Ta;
                float acc = 0.0F;
                for (uint32_t t = 0; t < hp; ++t) {
                    const float term = v[-(int)t] * w[t];
                    acc = acc + term;
                }
                const uint32_t nq = (Ta - hp) / 4u;
                const float* sq = sd + q0 - 4u;
                const float* wq = ws + mono_copy_base(Ta) + (h - 1u) * mono_copy_stride(Ta);
#pragma unroll 4
                for (uint32_t k = 0; k < nq; ++k) {
                    const float4 s4 = *reinterpret_cast<const float4*>(sq - 4u * k);
                    const float4 w4 = *reinterpret_cast<const float4*>(wq + 4u * k);
                    if (FAST) {
                        acc = __fmaf_rn(s4.w, w4.x, acc);
                        acc = __fmaf_rn(s4.z, w4.y, acc);
                        acc = __fmaf_rn(s4.y, w4.z, acc);
                        acc = __fmaf_rn(s4.x, w4.w, acc);
                    } else {
                        acc = acc + s4.w * w4.x;
                        acc = acc + s4.z * w4.y;
                        acc = acc + s4.y * w4.z;
                        acc = acc + s4.x * w4.w;
                    }
                }
                for (uint32_t t = hp + 4u * nq; t < Ta; ++t) {
                    const float term = v[-(int)t] * w[t];
                    acc = acc + term;
                }
                out[i] = acc * rx.gain;
            }
        }
        __syncthreads();
    }
}

unsigned persistent_grid(const void* kern, int threads, size_t shared, uint32_t nitems) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, shared);
    const uint32_t cap = (uint32_t)((per_sm > 0 ? per_sm : 1) * sms);
    return nitems < cap ? (nitems == 0 ? 1u : nitems) : cap;
}

// Dynamic plus static shared memory above 48 KB needs the opt-in attribute;
// it is set whenever a launch asks for more than it was last set to.
int32_t set_shared(const void* kern, size_t shared) {
    cudaFuncAttributes attr;
    if (int32_t st = cuda_status(cudaFuncGetAttributes(&attr, kern), "receiver kernel attributes")) return st;
    if ((size_t)attr.maxDynamicSharedSizeBytes >= shared) return RV_OK;
    return cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared),
                       "receiver kernel shared memory");
}

}  // namespace

int32_t launch_lerp_table(cudaStream_t s, const rv_cf32* taps, float2* lerped, uint32_t T, uint32_t P,
                          uint32_t period, uint32_t step_rem, uint32_t fd, float inv_fd) {
    const uint32_t total = period * T;
    const unsigned grid = (total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096;
    k_lerp_table<<<grid, 256, 0, s>>>(taps, lerped, T, P, period, step_rem, fd, inv_fd);
    return cuda_status(cudaGetLastError(), "lerp table");
}

int32_t launch_fine_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                            const float2* chan, uint32_t window_cap, uint32_t* queue, const uint32_t* dyn) {
    if (nitems == 0) return RV_OK;
    const size_t shared = (size_t)window_cap * sizeof(float2);
    if (int32_t st = set_shared((const void*)k_fine_batched, shared)) return st;
    const unsigned grid = persistent_grid((const void*)k_fine_batched, kRxThreads, shared, dyn ? ~0u : nitems);
    k_fine_batched<<<grid, kRxThreads, shared, s>>>(rxs, items, nitems, chan, window_cap, queue, dyn);
    return cuda_status(cudaGetLastError(), "fine batched");
}

uint32_t fine_unit_shared_budget() {
    static uint32_t budget = 0;
    if (budget == 0) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        // leave room for the kernel's static shared memory
        budget = (uint32_t)((optin > 2048 ? optin - 2048 : optin) / sizeof(float2));
    }
    return budget;
}

int32_t launch_fine_units(cudaStream_t s, const RxDev* rxs, const WorkItem* items, const FineUnit* units,
                          uint32_t nunits, const float2* chan, uint32_t shared_float2s, uint32_t* queue,
                          const uint32_t* dyn) {
    if (nunits == 0) return RV_OK;
    const size_t shared = (size_t)shared_float2s * sizeof(float2);
    if (int32_t st = set_shared((const void*)k_fine_units, shared)) return st;
    const unsigned grid = persistent_grid((const void*)k_fine_units, kUnitThreads, shared, dyn ? ~0u : nunits);
    k_fine_units<<<grid, kUnitThreads, shared, s>>>(rxs, items, units, nunits, chan, shared_float2s, queue, dyn);
    return cuda_status(cudaGetLastError(), "fine units");
}

int32_t launch_carrier_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                               const uint32_t* dyn) {
    if (nitems == 0) return RV_OK;
    k_carrier_batched<<<(nitems + 31) / 32, 32, 0, s>>>(rxs, items, nitems, dyn);
    return cuda_status(cudaGetLastError(), "carrier batched");
}

int32_t launch_detect_batched(cudaStream_t s, const RxDev* rxs, SpanList items, uint32_t nitems,
                              uint32_t window_cap, uint32_t* queue, const uint32_t* dyn, bool fast) {
    if (nitems == 0) return RV_OK;
    const size_t shared = (size_t)(window_cap + 4096u) * sizeof(float);  // window + DC weights
    const void* kern = fast ? (const void*)k_detect_batched<true> : (const void*)k_detect_batched<false>;
    if (int32_t st = set_shared(kern, shared)) return st;
    const unsigned grid = persistent_grid(kern, kRxThreads, shared, dyn ? ~0u : nitems);
    if (fast)
        k_detect_batched<true><<<grid, kRxThreads, shared, s>>>(rxs, items, nitems, window_cap, queue, dyn);
    else
        k_detect_batched<false><<<grid, kRxThreads, shared, s>>>(rxs, items, nitems, window_cap, queue, dyn);
    return cuda_status(cudaGetLastError(), "detect batched");
}

int32_t launch_audio_batched(cudaStream_t s, const RxDev* rxs, SpanList items, uint32_t nitems, float* audio,
                             uint32_t window_cap, uint32_t weights_cap, uint32_t* queue, const uint32_t* dyn, bool fast) {
    if (nitems == 0) return RV_OK;
    const size_t shared = (size_t)(window_cap + weights_cap) * sizeof(float);  // window, then the weights
    const void* kern = fast ? (const void*)k_audio_batched<true> : (const void*)k_audio_batched<false>;
    if (int32_t st = set_shared(kern, shared)) return st;
    const unsigned grid = persistent_grid(kern, kRxThreads, shared, dyn ? ~0u : nitems);
    if (fast)
        k_audio_batched<true><<<grid, kRxThreads, shared, s>>>(rxs, items, nitems, audio, window_cap, weights_cap, queue, dyn);
    else
        k_audio_batched<false><<<grid, kRxThreads, shared, s>>>(rxs, items, nitems, audio, window_cap, weights_cap, queue, dyn);
    return cuda_status(cudaGetLastError(), "audio batched");
}

}  // namespace rv
