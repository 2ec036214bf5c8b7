// Fused coarse chain: raw IQ ring -> convert -> polyphase branch FIR ->
// M-point FFT -> output phase correction -> channel-major ring, in one kernel.
//
// Computes exactly what the reference's three dispatches compute
// (convert_*_cf32.comp, pfb_branch.comp:98-149, pfb_fft.comp:274-363; twins
// core/dsp/convert.cpp, pfb_branch_reference.cpp:98-141,
// pfb_fft_reference.cpp:54-228): the same per-output operation order, the
// same butterfly arithmetic, so the channel ring is bit-identical to the
// plain path. What changes is the data movement:
//
//  * Branch FIR as register sliding windows. For branch r, block b and block
//    b + M/D share T-1 of their T input samples (the window advances by one
//    polyphase row). Each thread owns one (branch r, block phase) pair and
//    slides a T-sample window in registers, so every input sample is loaded
//    from HBM and converted exactly once per tile (plus a T-1 warm-up), and
//    each output costs T multiply-adds out of registers. Lanes of a warp own
//    consecutive r, so each load instruction is one coalesced run of samples.
//    The raw ring stays in its native width (4 B/sample for cs16), never
//    widened to cf32 in HBM.
//  * FFT in registers: radix-2 DIT stages taken three at a time inside one
//    thread (8 values), with one shared-memory transpose between groups; the
//    butterfly graph is the reference's, only visited in a different order.
//  * Output staged in shared memory so each channel's slots for a chunk of
//    blocks are written as one contiguous run.
//
// Per input sample the work is 2*T*M/D complex-by-real multiply-adds plus an
// (M/D)/M share of one M-point FFT; every multiply and add rounds separately
// (no FMA contraction, denormals flushed), as the reference twins require.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>

#include "common.cuh"
#include "receivers.cuh"
#include "revenant_gb300.h"

namespace rv {
int32_t validate_grid(const rv_grid_params* g);

namespace {

constexpr int kChunksPerTile = 8;

// One raw sample at unmasked ring position n, converted exactly as the plain
// convert kernel converts it; positions in the first lead_zero samples of
// block 0's support (before the stream began) read as 0.0.
// With a front-end table (in shared memory), the sample is then corrected
// with the parameters of the run it arrived in, as the plain path corrects a
// run's samples in place after converting them (core/shaders/iq_correct.comp).
template <int FMT>
__device__ __forceinline__ float2 convert_sample(const uint32_t* __restrict__ raw, uint32_t pos);

template <int FMT, bool FE>
__device__ __forceinline__ float2 load_sample(const uint32_t* __restrict__ raw, uint32_t n, const rv_coarse_params& p,
                                              uint32_t window_start, const FrontEndTable* fe) {
    const uint32_t rel = n - window_start;
    if (rel < p.lead_zero) return make_float2(0.0F, 0.0F);
    const float2 v = convert_sample<FMT>(raw, n & p.ring_mask);
    if (!FE) return v;
    uint32_t k = fe->count - 1u;
    while (k > 0u && rel < fe->e[k].rel_start) --k;
    const FrontEndEntry& e = fe->e[k];
    if (!e.on) return v;
    const float i = v.x - e.dc_i;
    const float q_dc = v.y - e.dc_q;
    const float a = e.cross * i;
    const float b = e.scale * q_dc;
    return make_float2(i, a + b);
}

template <int FMT>
__device__ __forceinline__ float2 convert_sample(const uint32_t* __restrict__ raw, uint32_t pos) {
    // a cf32 ring (already converted, corrected and excised) is read as is
    if (FMT == kFormatCf32Ring) return __ldg(reinterpret_cast<const float2*>(raw) + pos);
    return convert_raw<FMT>(raw, pos);
}

// acc += s * c for both components: a rounded multiply then a rounded add per
// component (packed f32x2 forms were measured not to reproduce the scalar
// rounding bit for bit, so they are not used).
__device__ __forceinline__ void mac(float2& acc, float2 s, float c) {
    acc.x = acc.x + s.x * c;
    acc.y = acc.y + s.y * c;
}

template <int L>
__device__ __forceinline__ uint32_t brev_c(uint32_t v) {
    return __brev(v) >> (32 - L);
}

template <int M>
struct Log2 {
    static constexpr int value = (M <= 1) ? 0 : 1 + Log2<M / 2>::value;
};
template <>
struct Log2<1> {
    static constexpr int value = 0;
};

// Position of local element u of FFT thread t when bit group g (bits
// [3g, 3g+3)) is held in registers.
__device__ __forceinline__ uint32_t group_pos(uint32_t t, uint32_t u, int g) {
    const uint32_t lo_mask = (1u << (3 * g)) - 1u;
    return (t & lo_mask) | (u << (3 * g)) | ((t >> (3 * g)) << (3 * g + 3));
}

template <int M, int T, int D, int FMT, int S, bool FE>
__global__ void __launch_bounds__(M*(M / D) * S)
k_coarse(const uint32_t* __restrict__ raw, const float* __restrict__ taps, const rv_cf32* __restrict__ tw_g,
         rv_cf32* __restrict__ ring, rv_coarse_params p_arg, uint32_t tiles_arg, const rv_coarse_params* dyn,
         const FrontEndTable* fe_g) {
    constexpr int P = M / D;          // block phases sharing no samples
    constexpr int NT = M * P * S;     // threads
    constexpr int CB = T * P;         // blocks per chunk per sub-stream
    constexpr int NB = CB * kChunksPerTile;
    constexpr int TILE = S * NB;
    constexpr int L = Log2<M>::value;
    static_assert(L % 3 == 0, "fused coarse kernel holds three FFT stages per register group");
    constexpr int G = L / 3;          // register groups of three stages
    constexpr int FT = M / 8;         // FFT threads per block
    constexpr int TASKS = S * CB * FT;
    constexpr int ROUNDS = (TASKS + NT - 1) / NT;
    // a launch captured in a CUDA graph reads this run's parameters from
    // device memory; a direct launch has them as arguments
    const rv_coarse_params p = dyn != nullptr ? *dyn : p_arg;
    const uint32_t tiles = dyn != nullptr ? (p.block_count + (uint32_t)TILE - 1u) / (uint32_t)TILE : tiles_arg;

    extern __shared__ float2 smem[];
    float2* twd = smem;               // [M]
    float2* A = twd + M;              // [S*CB][M] branch outputs, then transpose scratch
    float2* B = A + S * CB * M;       // [M][S*CB] channel-major staging

    const uint32_t tid = threadIdx.x;
    const uint32_t window_start = p.base_offset - (uint32_t)(M * T - 1);
    __shared__ FrontEndTable fe_s[1];
    if (FE) {
        for (uint32_t i = threadIdx.x; i < sizeof(FrontEndTable) / 4u; i += blockDim.x)
            reinterpret_cast<uint32_t*>(fe_s)[i] = reinterpret_cast<const uint32_t*>(fe_g)[i];
    }
    const FrontEndTable* fe = fe_s;  // read only when FE; visible after the barrier below
    for (uint32_t i = tid; i < (uint32_t)M; i += NT) twd[i] = ld_cf32(&tw_g[i]);

    const uint32_t r = tid % M;
    const uint32_t par = (tid / M) % P;
    const uint32_t s = tid / (M * P);
    float h[T];
#pragma unroll
    for (int q = 0; q < T; ++q) h[q] = taps[q * M + r];
    __syncthreads();

    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t tile0 = tile * (uint32_t)TILE;
        // ring position of this thread's q = 0 sample for its first block
        const uint32_t n0 = p.base_offset + (tile0 + s * NB + par) * (uint32_t)D - r;
        float2 win[T];
#pragma unroll
        for (int q = 1; q < T; ++q) win[T - q] = load_sample<FMT, FE>(raw, n0 - (uint32_t)(q * M), p, window_start, fe);

        for (int c = 0; c < kChunksPerTile; ++c) {
            // ---- branch FIR: T steps, window slot of sample q at step i is (i - q) mod T
#pragma unroll
            for (int i = 0; i < T; ++i) {
                const uint32_t g = (uint32_t)(c * T + i);
                win[i] = load_sample<FMT, FE>(raw, n0 + g * (uint32_t)M, p, window_start, fe);
                float2 acc = make_float2(0.0F, 0.0F);
#pragma unroll
                for (int q = 0; q < T; ++q) mac(acc, win[(i - q + T) % T], h[q]);
                const uint32_t bl = (uint32_t)i * P + par;
                A[(s * CB + bl) * M + ((M - r) & (M - 1u))] = acc;
            }
            __syncthreads();

            // ---- FFT, 8 values per thread, three stages per register group
#pragma unroll 1
            for (int round = 0; round < ROUNDS; ++round) {
                const uint32_t task = (uint32_t)round * NT + tid;
                const bool valid = task < (uint32_t)TASKS;
                const uint32_t blk = valid ? task / FT : 0u;
                const uint32_t t = task % FT;
                float2* a = A + blk * M;
                float2 v[8];
                if (valid) {
#pragma unroll
                    for (int u = 0; u < 8; ++u) v[u] = a[brev_c<L>(group_pos(t, u, 0))];
                }
#pragma unroll
                for (int grp = 0; grp < G; ++grp) {
                    if (grp > 0) {
                        __syncwarp();
                        if (valid) {
#pragma unroll
                            for (int u = 0; u < 8; ++u) a[group_pos(t, u, grp - 1)] = v[u];
                        }
                        __syncwarp();
                        if (valid) {
#pragma unroll
                            for (int u = 0; u < 8; ++u) v[u] = a[group_pos(t, u, grp)];
                        }
                    }
#pragma unroll
                    for (int l = 0; l < 3; ++l) {
                        const int st = 3 * grp + l;
                        const uint32_t half = 1u << st;
                        const uint32_t step = (uint32_t)M >> (st + 1);
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            if (u & (1 << l)) continue;
                            const uint32_t j = group_pos(t, (uint32_t)u, grp) & (half - 1u);
                            butterfly(v[u], v[u | (1 << l)], twd[j * step]);
                        }
                    }
                }
                if (valid) {
                    const uint32_t sb = blk / CB, bl = blk % CB;
                    const uint32_t m_abs = p.block_base + tile0 + sb * NB + (uint32_t)c * CB + bl;
                    const uint32_t dm = ((m_abs & (M - 1u)) * (uint32_t)D) & (M - 1u);
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const uint32_t k = group_pos(t, u, G - 1);
                        float2 val = v[u];
                        if (D != M) val = cmul(val, twd[(k * dm) & (M - 1u)]);
                        B[k * (S * CB) + blk] = val;
                    }
                }
            }
            __syncthreads();

            // ---- write-out: each channel's run of S*CB slots
            for (uint32_t e = tid; e < (uint32_t)(M * S * CB); e += NT) {
                const uint32_t k = e / (S * CB), blk = e % (S * CB);
                const uint32_t sb = blk / CB, bl = blk % CB;
                const uint32_t m_local = tile0 + sb * NB + (uint32_t)c * CB + bl;
                if (m_local < p.block_count) {
                    const uint32_t slot = (p.block_base + m_local) & p.out_ring_mask;
                    st_cf32(&ring[(uint64_t)k * p.out_ring_blocks + slot], B[e]);
                }
            }
        }
    }
}

template <int M, int T, int D, int FMT, int S, bool FE>
int32_t launch(cudaStream_t stream, const uint32_t* raw, const float* taps, const rv_cf32* tw, rv_cf32* ring,
               const rv_coarse_params& p, const rv_coarse_params* dyn, const FrontEndTable* fe) {
    constexpr int P = M / D, NT = M * P * S, CB = T * P;
    constexpr int TILE = S * CB * kChunksPerTile;
    const size_t shared = sizeof(float2) * (M + 2 * S * CB * M);
    auto kern = k_coarse<M, T, D, FMT, S, FE>;
    if (int32_t st = ensure_shared((const void*)kern, shared, "coarse shared")) return st;
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (int32_t st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, shared),
                                 "coarse occupancy"))
        return st;
    const int max_grid = (per_sm > 0 ? per_sm : 1) * sms;
    const uint32_t tiles = (p.block_count + TILE - 1) / TILE;
    // captured: the full resident grid, for whatever block count the run has
    const uint32_t grid = dyn != nullptr ? (uint32_t)max_grid : (tiles < (uint32_t)max_grid ? tiles : (uint32_t)max_grid);
    kern<<<grid, NT, shared, stream>>>(raw, taps, tw, ring, p, tiles, dyn, fe);
    return cuda_status(cudaGetLastError(), "coarse_fused launch");
}

// ---- any grid of up to 1024 channels and M/D <= 4 (C2's M = 1024, D = 512,
// T = 16 among them), grid sizes given at run time. A CTA takes batches of
// kWideB * P consecutive blocks (P = M/D block phases), one thread per branch
// r. Block b + P is one polyphase row later than block b, so for each phase
// the thread loads its T - 1 older samples once and then one new sample per
// block, keeping the window in registers (each raw sample is read and
// converted once per phase and batch, plus the warm-up). Branch outputs go
// straight to their bit-reversed slots in shared memory; the batch's
// transforms then run the reference's radix-2 DIT stages together (the same
// butterflies as the plain kernel), and each channel's slots of the batch are
// phase-corrected and written as one contiguous run of the channel-major
// ring: every output's operations as in the plain path.
constexpr uint32_t kWideB = 4;  // consecutive blocks of one phase in a batch

template <int T, int FMT, bool FE>
__global__ void __launch_bounds__(1024, 1)
k_coarse_wide(const uint32_t* __restrict__ raw, const float* __restrict__ taps, const rv_cf32* __restrict__ tw_g,
              rv_cf32* __restrict__ ring, rv_coarse_params p_arg, uint32_t M, uint32_t D, uint32_t stages,
              const rv_coarse_params* dyn, const FrontEndTable* fe_g) {
    const rv_coarse_params p = dyn != nullptr ? *dyn : p_arg;
    const uint32_t P = M / D, NBB = kWideB * P;  // blocks a batch
    const uint32_t pitch = M + 1u;               // transform rows, padded against bank conflicts
    const uint32_t batches = (p.block_count + NBB - 1u) / NBB;
    extern __shared__ float2 smem[];
    float2* twd = smem;   // [M]
    float2* x = twd + M;  // [NBB][pitch] the transforms
    __shared__ FrontEndTable fe_s[1];
    if (FE) {
        for (uint32_t i = threadIdx.x; i < sizeof(FrontEndTable) / 4u; i += blockDim.x)
            reinterpret_cast<uint32_t*>(fe_s)[i] = reinterpret_cast<const uint32_t*>(fe_g)[i];
    }
    const FrontEndTable* fe = fe_s;
    for (uint32_t i = threadIdx.x; i < M; i += blockDim.x) twd[i] = ld_cf32(&tw_g[i]);
    const uint32_t r = threadIdx.x;  // blockDim.x == M
    const uint32_t slot_in = brev((M - r) & (M - 1u), stages);
    const uint32_t window_start = p.base_offset - (M * (uint32_t)T - 1u);
    float h[T];
#pragma unroll
    for (int q = 0; q < T; ++q) h[q] = taps[(uint32_t)q * M + r];
    __syncthreads();
    for (uint32_t batch = blockIdx.x; batch < batches; batch += gridDim.x) {
        const uint32_t blk0 = batch * NBB;
        const uint32_t nb = (p.block_count - blk0 < NBB) ? p.block_count - blk0 : NBB;
        // ---- branch FIR, phase by phase: blocks blk0 + ph + j P, j < kWideB
        for (uint32_t ph = 0; ph < P; ++ph) {
            const uint32_t n0 = p.base_offset + (blk0 + ph) * D - r;  // newest sample (q = 0) of j = 0
            float2 win[T];
#pragma unroll
            for (int q = 1; q < T; ++q) win[T - q] = load_sample<FMT, FE>(raw, n0 - (uint32_t)q * M, p, window_start, fe);
#pragma unroll
            for (int j = 0; j < (int)kWideB; ++j) {
                win[j] = load_sample<FMT, FE>(raw, n0 + (uint32_t)j * M, p, window_start, fe);
                float2 acc = make_float2(0.0F, 0.0F);
#pragma unroll
                for (int q = 0; q < T; ++q) mac(acc, win[(j - q + T) % T], h[q]);
                const uint32_t lb = ph + (uint32_t)j * P;  // block within the batch
                if (lb < nb) x[lb * pitch + slot_in] = acc;
            }
        }
        __syncthreads();
        // ---- the batch's transforms, each stage for all of them
        const uint32_t half_m = M >> 1;  // butterflies a transform a stage (a power of two)
        for (uint32_t st = 0; st < stages; ++st) {
            const uint32_t half = 1u << st, step = M >> (st + 1u);
            for (uint32_t u = r; u < nb * half_m; u += M) {
                float2* xb = x + (u >> (stages - 1u)) * pitch;
                const uint32_t bf = u & (half_m - 1u);
                const uint32_t jj = bf & (half - 1u);
                const uint32_t ia = ((bf >> st) << (st + 1u)) + jj;
                butterfly(xb[ia], xb[ia + half], twd[jj * step]);
            }
            __syncthreads();
        }
        // ---- phase correction and write-out: each channel's slots together
        // (NBB a power of two: kWideB times a power-of-two P)
        const uint32_t nbb_log2 = 31u - (uint32_t)__clz(NBB);
        for (uint32_t e = r; e < M * NBB; e += M) {
            const uint32_t k = e >> nbb_log2, lb = e & (NBB - 1u);
            if (lb >= nb) continue;
            const uint32_t m_abs = p.block_base + blk0 + lb;
            const uint32_t dm = ((m_abs & (M - 1u)) * D) & (M - 1u);
            float2 v = x[lb * pitch + k];
            if (D != M) v = cmul(v, twd[(k * dm) & (M - 1u)]);
            st_cf32(&ring[(uint64_t)k * p.out_ring_blocks + (m_abs & p.out_ring_mask)], v);
        }
        __syncthreads();  // the transforms are read before the next batch's branch outputs land
    }
}

bool coarse_wide_supported(const rv_grid_params& g) {
    const uint32_t M = g.channels;
    return M >= 32u && M <= 1024u && (M & (M - 1u)) == 0u && g.decimation != 0u && M % g.decimation == 0u &&
           M / g.decimation <= 4u && (g.taps_per_branch == 16u || g.taps_per_branch == 17u);
}

template <int T, int FMT, bool FE>
int32_t launch_wide(cudaStream_t stream, const rv_grid_params& g, const uint32_t* raw, const float* taps,
                    const rv_cf32* tw, rv_cf32* ring, const rv_coarse_params& p, const rv_coarse_params* dyn,
                    const FrontEndTable* fe) {
    const uint32_t M = g.channels, D = g.decimation, P = M / D;
    uint32_t stages = 0;
    while ((1u << stages) < M) ++stages;
    const size_t shared = sizeof(float2) * ((size_t)M + (size_t)kWideB * P * (M + 1u));
    auto kern = k_coarse_wide<T, FMT, FE>;
    if (int32_t st = ensure_shared((const void*)kern, shared, "coarse wide shared")) return st;
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (int32_t st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)M, shared),
                                 "coarse wide occupancy"))
        return st;
    const uint32_t max_grid = (uint32_t)(per_sm > 0 ? per_sm : 1) * (uint32_t)sms;
    const uint32_t NBB = kWideB * P;
    const uint32_t batches = (p.block_count + NBB - 1u) / NBB;
    const uint32_t grid = dyn != nullptr ? max_grid : (batches < max_grid ? batches : max_grid);
    kern<<<grid, M, shared, stream>>>(raw, taps, tw, ring, p, M, D, stages, dyn, fe);
    return cuda_status(cudaGetLastError(), "coarse wide launch");
}

template <int T>
int32_t dispatch_wide(cudaStream_t stream, const rv_grid_params& g, int32_t format, const uint32_t* raw,
                      const float* taps, const rv_cf32* tw, rv_cf32* ring, const rv_coarse_params& p,
                      const rv_coarse_params* dyn, const FrontEndTable* fe) {
    if (format == RV_FORMAT_CS16)
        return fe ? launch_wide<T, RV_FORMAT_CS16, true>(stream, g, raw, taps, tw, ring, p, dyn, fe)
                  : launch_wide<T, RV_FORMAT_CS16, false>(stream, g, raw, taps, tw, ring, p, dyn, fe);
    if (format == RV_FORMAT_CU8)
        return fe ? launch_wide<T, RV_FORMAT_CU8, true>(stream, g, raw, taps, tw, ring, p, dyn, fe)
                  : launch_wide<T, RV_FORMAT_CU8, false>(stream, g, raw, taps, tw, ring, p, dyn, fe);
    if (format == kFormatCf32Ring && fe == nullptr)
        return launch_wide<T, kFormatCf32Ring, false>(stream, g, raw, taps, tw, ring, p, dyn, fe);
    return set_error_fmt(RV_ERR_UNSUPPORTED, "coarse_fused: format %d", format);
}

// Source samples [from, from + count) of the raw ring converted into the cf32
// ring at the same slots, each corrected with the parameters of the run it
// arrived in (the table's entries are relative to window_start), exactly as
// the coarse kernel converts and corrects the samples it loads.
template <int FMT, bool FE>
__global__ void k_convert_ring(const uint32_t* __restrict__ raw, uint32_t mask, uint32_t from, uint32_t count,
                               uint32_t window_start, const FrontEndTable* fe_g, float2* __restrict__ clean) {
    __shared__ FrontEndTable fe_s[1];
    if (FE) {
        for (uint32_t i = threadIdx.x; i < sizeof(FrontEndTable) / 4u; i += blockDim.x)
            reinterpret_cast<uint32_t*>(fe_s)[i] = reinterpret_cast<const uint32_t*>(fe_g)[i];
        __syncthreads();
    }
    rv_coarse_params p{};
    p.ring_mask = mask;
    p.lead_zero = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t n = from + i;
        clean[n & mask] = load_sample<FMT, FE>(raw, n, p, window_start, fe_s);
    }
}

template <int FMT>
int32_t convert_ring(cudaStream_t s, const uint32_t* raw, uint32_t mask, uint32_t from, uint32_t count,
                     uint32_t window_start, const FrontEndTable* fe, float2* clean) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t grid = std::min<uint32_t>((count + 255u) / 256u, (uint32_t)(sms > 0 ? sms : 1) * 8u);
    if (fe)
        k_convert_ring<FMT, true><<<grid, 256, 0, s>>>(raw, mask, from, count, window_start, fe, clean);
    else
        k_convert_ring<FMT, false><<<grid, 256, 0, s>>>(raw, mask, from, count, window_start, fe, clean);
    return cuda_status(cudaGetLastError(), "convert_ring launch");
}

}  // namespace

int32_t launch_convert_ring(cudaStream_t stream, int32_t format, const void* raw, uint32_t mask, uint32_t from,
                            uint32_t count, uint32_t window_start, const FrontEndTable* fe, rv_cf32* clean) {
    if (count == 0) return RV_OK;
    const uint32_t* w = static_cast<const uint32_t*>(raw);
    float2* out = reinterpret_cast<float2*>(clean);
    if (format == RV_FORMAT_CS16) return convert_ring<RV_FORMAT_CS16>(stream, w, mask, from, count, window_start, fe, out);
    if (format == RV_FORMAT_CU8) return convert_ring<RV_FORMAT_CU8>(stream, w, mask, from, count, window_start, fe, out);
    return set_error_fmt(RV_ERR_UNSUPPORTED, "convert_ring: format %d", format);
}

// Whether a fused kernel is instantiated for the grid.
bool coarse_fused_supported(const rv_grid_params& g) {
    return (g.channels == 64 && g.taps_per_branch == 17 && g.decimation == 32) ||
           (g.channels == 8 && g.taps_per_branch == 17 && g.decimation == 4) ||
           (g.channels == 64 && g.taps_per_branch == 17 && g.decimation == 64) || coarse_wide_supported(g);
}

// Dispatch over the instantiated grids. Returns RV_ERR_UNSUPPORTED for a
// grid this build has no fused kernel for (the plain kernels cover it).
int32_t launch_coarse_fused(cudaStream_t stream, const rv_grid_params& g, int32_t format, const rv_coarse_params& p,
                            const void* raw, const float* taps, const rv_cf32* tw, rv_cf32* ring,
                            const rv_coarse_params* dyn, const FrontEndTable* fe) {
    const uint32_t* w = static_cast<const uint32_t*>(raw);
#define RV_COARSE_CASE(MM, TT, DD, SS)                                                                    \
    if (g.channels == MM && g.taps_per_branch == TT && g.decimation == DD) {                             \
        if (format == RV_FORMAT_CS16)                                                                    \
            return fe ? launch<MM, TT, DD, RV_FORMAT_CS16, SS, true>(stream, w, taps, tw, ring, p, dyn, fe)   \
                      : launch<MM, TT, DD, RV_FORMAT_CS16, SS, false>(stream, w, taps, tw, ring, p, dyn, fe); \
        if (format == RV_FORMAT_CU8)                                                                     \
            return fe ? launch<MM, TT, DD, RV_FORMAT_CU8, SS, true>(stream, w, taps, tw, ring, p, dyn, fe)    \
                      : launch<MM, TT, DD, RV_FORMAT_CU8, SS, false>(stream, w, taps, tw, ring, p, dyn, fe);  \
        if (format == kFormatCf32Ring && fe == nullptr)                                                  \
            return launch<MM, TT, DD, kFormatCf32Ring, SS, false>(stream, w, taps, tw, ring, p, dyn, fe);   \
    }
    RV_COARSE_CASE(64, 17, 32, 1)
    RV_COARSE_CASE(8, 17, 4, 8)
    RV_COARSE_CASE(64, 17, 64, 2)
#undef RV_COARSE_CASE
    if (coarse_wide_supported(g)) {
        if (g.taps_per_branch == 16u) return dispatch_wide<16>(stream, g, format, w, taps, tw, ring, p, dyn, fe);
        return dispatch_wide<17>(stream, g, format, w, taps, tw, ring, p, dyn, fe);
    }
    return set_error_fmt(RV_ERR_UNSUPPORTED,
                         "coarse_fused: no fused kernel for M=%u T=%u D=%u format %d in this build (use the plain launches)",
                         g.channels, g.taps_per_branch, g.decimation, format);
}

int32_t validate_coarse(const rv_grid_params* g, int32_t format, const rv_coarse_params* p, uint64_t raw_bytes,
                        uint64_t taps_len, uint64_t tw_len, uint64_t ring_len) {
    if (int32_t st = validate_grid(g)) return st;
    if (format != RV_FORMAT_CS16 && format != RV_FORMAT_CU8)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "coarse_fused: format %d (cs16 and cu8 are fused)", format);
    const uint32_t M = g->channels, T = g->taps_per_branch, D = g->decimation;
    const uint64_t cap = (uint64_t)p->ring_mask + 1u;
    if ((cap & (uint64_t)p->ring_mask) != 0 || cap < 2)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: ring_mask %u is not a power of two minus one", p->ring_mask);
    const uint64_t need_bytes = format == RV_FORMAT_CS16 ? cap * 4u : cap * 2u;
    if (raw_bytes < need_bytes)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: raw ring holds %llu bytes, mask implies %llu",
                             (unsigned long long)raw_bytes, (unsigned long long)need_bytes);
    if (taps_len != (uint64_t)M * T) return set_error_fmt(RV_ERR_INVALID, "coarse_fused: wants %u taps", M * T);
    if (tw_len != M) return set_error_fmt(RV_ERR_INVALID, "coarse_fused: wants %u twiddles", M);
    if (p->block_count == 0) return RV_OK;
    const uint64_t span = (uint64_t)M * T + (uint64_t)(p->block_count - 1u) * D;
    if (span > cap)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: needs %llu samples of history, ring capacity is %llu",
                             (unsigned long long)span, (unsigned long long)cap);
    if (p->lead_zero > M * T - 1u)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: lead_zero %u exceeds M*T - 1 = %u", p->lead_zero, M * T - 1u);
    if (!is_pow2(p->out_ring_blocks) || p->out_ring_mask != p->out_ring_blocks - 1u)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: out_ring_blocks must be a power of two and out_ring_mask one less");
    if (p->block_count > p->out_ring_blocks)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: %u blocks overrun a %u-block ring", p->block_count,
                             p->out_ring_blocks);
    if (ring_len < (uint64_t)M * p->out_ring_blocks)
        return set_error_fmt(RV_ERR_INVALID, "coarse_fused: channel ring too short");
    return RV_OK;
}

}  // namespace rv

extern "C" int32_t rv_coarse_fused(void* stream, const rv_grid_params* grid, int32_t format,
                                   const rv_coarse_params* params, const void* raw_ring_dev, uint64_t raw_ring_bytes,
                                   const float* taps_dev, uint64_t taps_len, const rv_cf32* twiddles_dev,
                                   uint64_t twiddles_len, rv_cf32* channel_ring_dev, uint64_t channel_ring_len) {
    if (grid == nullptr || params == nullptr || raw_ring_dev == nullptr || taps_dev == nullptr ||
        twiddles_dev == nullptr || channel_ring_dev == nullptr)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_coarse_fused: NULL argument");
    if (int32_t st = rv::validate_coarse(grid, format, params, raw_ring_bytes, taps_len, twiddles_len, channel_ring_len))
        return st;
    if (params->block_count == 0) return rv::clear_error();
    if (((uintptr_t)raw_ring_dev & 3u) != 0)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_coarse_fused: raw ring is not 4-byte aligned");
    if (int32_t st = rv::launch_coarse_fused(reinterpret_cast<cudaStream_t>(stream), *grid, format, *params,
                                             raw_ring_dev, taps_dev, twiddles_dev, channel_ring_dev, nullptr, nullptr))
        return st;
    return rv::clear_error();
}
