// C4's split-precision channelizer DFT on the 5th-generation tensor cores.
//
// rv_pfb_fft's transform (core/dsp/pfb_fft_reference.cpp:54-102 transform_block:
// Y[k] = sum_n y[n] W^(kn), W = exp(-2 pi i / M), then the phase correction
// W^(k dm), dm = ((m & (M-1)) D) & (M-1), and the channel-major scatter) for
// M = 4096, computed as the four-step factorisation M = 64 x 64:
//
//   n = 64 n1 + n2, k = k1 + 64 k2
//   Z[k1][n2]  = sum_n1 F[k1][n1] y'[64 n1 + n2]          (GEMM 1)
//   Z'[k1][n2] = Z[k1][n2] W^(k1 n2)                        (twiddle, FP32)
//   Y[k1 + 64 k2] = sum_n2 F[k2][n2] Z'[k1][n2]            (GEMM 2)
//
// with F the 64-point DFT matrix and y'[n] = y[(n - dm) mod M] (the phase
// correction W^(k dm) folded in as an exact rotation of the input). Each
// complex GEMM is one real GEMM of M = 128 rows ([Re | Im] of the output
// index), K = 128 ([Re | Im] of the summed index) and N = 128 columns (two
// blocks x 64) on tcgen05.mma kind::f16 with FP32 accumulators in tensor
// memory. Operands are split hi + lo (FP16 or BF16): x = hi + lo 2^-s, and
//   acc0 = A_hi B_hi,  acc1 = A_hi B_lo + A_lo B_hi,  result = acc0 + acc1 2^-s,
// so each product carries about twice the input type's significand. For FP16
// each block is scaled by a power of two (exact) so its largest component sits
// just below 2^14 before splitting, and GEMM 2's operand by 2^-6, keeping every
// hi and lo part in FP16's normal range; the scales are undone on output.
//
// One CTA per SM (four warps, 193 KB of shared memory), persistent over pairs
// of blocks. Operands are written to shared memory by the threads in the
// canonical no-swizzle K-major layout (8-row x 16-byte core matrices); thread
// 0 issues the MMAs and commits them to an mbarrier; every warp reads its 32
// TMEM lanes back with tcgen05.ld. Every mbarrier wait is bounded: a wait that
// runs out sets an error flag the host reads, and the CTA frees its TMEM and
// returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace rv {
namespace {

constexpr uint32_t kM = 4096;
constexpr uint32_t kRadix = 64;
constexpr uint32_t kPair = 2;                       // blocks per tile
constexpr uint32_t kRows = 128;                     // GEMM M: [Re | Im] x 64
constexpr uint32_t kK = 128;                        // GEMM K: [Re | Im] x 64
constexpr uint32_t kCols = kPair * kRadix;          // GEMM N
constexpr uint32_t kOperand = kRows * kK * 2;       // one 16-bit operand: 32 KB
constexpr uint32_t kPitch = kCols + 1;              // FP32 staging row pitch
constexpr uint32_t kStageBytes = kRows * kPitch * 4;  // 66,048
constexpr uint32_t kOffA = 0;                       // A_hi, A_lo
constexpr uint32_t kOffX = 2 * kOperand;            // B1_hi, B1_lo | FP32 staging
constexpr uint32_t kOffB2 = kOffX + kStageBytes;    // B2_hi, B2_lo
constexpr uint32_t kOffMisc = kOffB2 + 2 * kOperand;
constexpr uint32_t kSmemBytes = kOffMisc + 64;
constexpr uint32_t kThreads = 128;
constexpr uint32_t kTmemCols = 256;                 // acc0 at column 0, acc1 at 128
constexpr uint32_t kWaitLimit = 1u << 20;

__device__ uint32_t g_dft_timeouts;

// Element (r, k) of a 128 x 128 K-major operand: core matrix (r/8, k/8) at
// ((r/8) * 16 + k/8) * 128 bytes, row r%8 at 16 bytes each. K-adjacent core
// matrices are 128 bytes apart (LBO), 8-row groups 2048 (SBO).
__device__ __forceinline__ uint32_t core_offset(uint32_t r, uint32_t k) {
    return ((r >> 3) * (kK / 8) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(2048u >> 4) << 32) |
           (1ull << 46);  // descriptor version 1; base offset 0; no swizzle
}

// kind::f16, FP32 accumulate, A and B K-major, M = 128, N = 128.
template <int P>
__host__ __device__ constexpr uint32_t instr_desc() {
    return (1u << 4) | ((uint32_t)P << 7) | ((uint32_t)P << 10) | ((kCols >> 3) << 17) | ((kRows >> 4) << 24);
}

template <int P>
struct Split;
template <>
struct Split<RV_DFT_FP16> {
    static constexpr float kLo = 2048.0F, kInvLo = 1.0F / 2048.0F;
    __device__ static float round(float x) { return __half2float(__float2half_rn(x)); }
    __device__ static uint32_t pack(float a, float b) {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
};
template <>
struct Split<RV_DFT_BF16> {
    static constexpr float kLo = 256.0F, kInvLo = 1.0F / 256.0F;
    __device__ static float round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
    __device__ static uint32_t pack(float a, float b) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
};

// Eight values of one operand row split and stored as two 16-byte runs (hi
// into `hi`, lo into `lo`) at k = 8j .. 8j + 7.
template <int P>
__device__ __forceinline__ void store_split8(uint8_t* hi, uint8_t* lo, uint32_t r, uint32_t k0, const float* v) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float h0 = Split<P>::round(v[2 * i]), h1 = Split<P>::round(v[2 * i + 1]);
        h[i] = Split<P>::pack(h0, h1);
        l[i] = Split<P>::pack((v[2 * i] - h0) * Split<P>::kLo, (v[2 * i + 1] - h1) * Split<P>::kLo);
    }
    const uint32_t off = core_offset(r, k0);
    *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool wait_parity(uint32_t mbar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// The two accumulators of this thread's row combined into the FP32 staging
// row: acc0 + acc1 2^-s, times `scale`.
template <int P>
__device__ __forceinline__ void drain_row(uint32_t tmem, uint32_t row, float* stage, float scale) {
    const uint32_t lane_base = tmem + (((row >> 5) * 32u) << 16);
    for (uint32_t c = 0; c < kCols; c += 32) {
        float a[32], b[32];
        tmem_ld32(lane_base + c, a);
        tmem_ld32(lane_base + kCols + c, b);
#pragma unroll
        for (int i = 0; i < 32; ++i) stage[row * kPitch + c + i] = (a[i] + b[i] * Split<P>::kInvLo) * scale;
    }
}

// Both GEMMs of one stage: 8 K-steps of 16 for each of the three products.
template <int P>
__device__ __forceinline__ void issue_gemm(uint32_t tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi, uint32_t b_lo,
                                           uint32_t mbar) {
    fence_after();
    constexpr uint32_t idesc = instr_desc<P>();
    for (uint32_t s = 0; s < kK / 16; ++s) mma(tmem, smem_desc(a_hi + 256u * s), smem_desc(b_hi + 256u * s), idesc, s);
    for (uint32_t s = 0; s < kK / 16; ++s)
        mma(tmem + kCols, smem_desc(a_hi + 256u * s), smem_desc(b_lo + 256u * s), idesc, s);
    for (uint32_t s = 0; s < kK / 16; ++s)
        mma(tmem + kCols, smem_desc(a_lo + 256u * s), smem_desc(b_hi + 256u * s), idesc, 1u);
    commit(mbar);
}

template <int P>
__global__ void __launch_bounds__(kThreads, 1)
k_dft_tc(const float2* __restrict__ branch, const float2* __restrict__ tw, float2* __restrict__ out,
         rv_pfb_fft_params p) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* const a_hi = sm + kOffA;
    uint8_t* const a_lo = a_hi + kOperand;
    uint8_t* const x_hi = sm + kOffX;  // B1 (hi, lo), then the FP32 staging
    uint8_t* const x_lo = x_hi + kOperand;
    float* const stage = reinterpret_cast<float*>(sm + kOffX);
    uint8_t* const b2_hi = sm + kOffB2;
    uint8_t* const b2_lo = b2_hi + kOperand;
    uint64_t* const mbar = reinterpret_cast<uint64_t*>(sm + kOffMisc);
    uint32_t* const tmem_slot = reinterpret_cast<uint32_t*>(sm + kOffMisc + 8);
    uint32_t* const abort_flag = reinterpret_cast<uint32_t*>(sm + kOffMisc + 12);
    float* const block_max = reinterpret_cast<float*>(sm + kOffMisc + 16);  // [kPair][2 warps]
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t mbar_addr = smem_addr(mbar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_addr));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort_flag = 0;
    }
    // A = F in real block form, the same for both stages: row r = [Re | Im]
    // of the output index, column k = [Re | Im] of the summed index.
    {
        const uint32_t r = tid, kr = r & 63u;
        for (uint32_t j = 0; j < kK / 8; ++j) {
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint32_t k = 8u * j + (uint32_t)i, kn = k & 63u;
                const float2 f = tw[(kRadix * kr * kn) & (kM - 1u)];
                v[i] = (r < 64u) ? (k < 64u ? f.x : -f.y) : (k < 64u ? f.y : f.x);
            }
            store_split8<P>(a_hi, a_lo, r, 8u * j, v);
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    const uint32_t tiles = (p.block_count + kPair - 1u) / kPair;
    uint32_t parity = 0;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t b0 = tile * kPair;
        // this thread's B1 row: block `blk` of the pair, n2
        const uint32_t blk = tid >> 6, n2 = tid & 63u, b = b0 + blk;
        const bool valid = b < p.block_count;
        const float2* y = branch + (uint64_t)(valid ? b : b0) * kM;
        const uint32_t m_abs = p.block_base + b;
        const uint32_t dm = ((m_abs & (kM - 1u)) * p.decimation) & (kM - 1u);
        // the block's largest component, for the power-of-two scale
        float mx = 0.0F;
        if (valid)
            for (uint32_t n1 = 0; n1 < kRadix; ++n1) {
                const float2 v = y[(kRadix * n1 + n2 - dm) & (kM - 1u)];
                mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
        if (lane == 0) block_max[warp] = mx;
        __syncthreads();
        const float bmax = fmaxf(block_max[blk * 2], block_max[blk * 2 + 1]);
        int shift = 0;  // scale = 2^shift puts bmax in [2^13, 2^14)
        if (bmax > 0.0F) {
            const int e = (int)((__float_as_uint(bmax) >> 23) & 0xFFu) - 127;
            shift = 13 - e;
            shift = shift > 100 ? 100 : (shift < -100 ? -100 : shift);
        }
        const float scale_in = ldexpf(1.0F, shift);
        // B1 row (blk, n2): K = [Re | Im] of y'[64 n1 + n2], n1 = 0..63
        for (uint32_t j = 0; j < kRadix / 8; ++j) {
            float re[8], im[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint32_t n1 = 8u * j + (uint32_t)i;
                const float2 v = valid ? y[(kRadix * n1 + n2 - dm) & (kM - 1u)] : make_float2(0.0F, 0.0F);
                re[i] = v.x * scale_in;
                im[i] = v.y * scale_in;
            }
            store_split8<P>(x_hi, x_lo, tid, 8u * j, re);
            store_split8<P>(x_hi, x_lo, tid, kRadix + 8u * j, im);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) issue_gemm<P>(tmem, smem_addr(a_hi), smem_addr(a_lo), smem_addr(x_hi), smem_addr(x_lo), mbar_addr);
        if (!wait_parity(mbar_addr, parity)) atomicExch(abort_flag, 1u);
        parity ^= 1u;
        __syncthreads();
        if (*abort_flag) break;
        fence_after();
        // GEMM 1 out: row tid = [Re | Im] Z[k1], columns (blk, n2); times 2^-6
        drain_row<P>(tmem, tid, stage, 1.0F / 64.0F);
        fence_before();
        __syncthreads();
        // B2 row (blk, k1): K = [Re | Im] of Z'[k1][n2] = Z[k1][n2] W^(k1 n2)
        {
            const uint32_t k1 = tid & 63u, col0 = blk * kRadix;
            for (uint32_t j = 0; j < kRadix / 8; ++j) {
                float re[8], im[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const uint32_t c = 8u * j + (uint32_t)i;
                    const float zr = stage[k1 * kPitch + col0 + c], zi = stage[(64u + k1) * kPitch + col0 + c];
                    const float2 w = tw[(k1 * c) & (kM - 1u)];
                    re[i] = zr * w.x - zi * w.y;
                    im[i] = zr * w.y + zi * w.x;
                }
                store_split8<P>(b2_hi, b2_lo, tid, 8u * j, re);
                store_split8<P>(b2_hi, b2_lo, tid, kRadix + 8u * j, im);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0)
            issue_gemm<P>(tmem, smem_addr(a_hi), smem_addr(a_lo), smem_addr(b2_hi), smem_addr(b2_lo), mbar_addr);
        if (!wait_parity(mbar_addr, parity)) atomicExch(abort_flag, 1u);
        parity ^= 1u;
        __syncthreads();
        if (*abort_flag) break;
        fence_after();
        // GEMM 2 out: row tid = [Re | Im] Y[k1 + 64 k2] for k2, columns (blk, k1);
        // undo the scales: 2^6 2^-shift (this row's block differs per column
        // half, so the scale is applied on output)
        drain_row<P>(tmem, tid, stage, 64.0F);
        fence_before();
        __syncthreads();
        if (valid) {
            const float scale_out = ldexpf(1.0F, -shift);
            const uint32_t k2 = tid & 63u, slot = m_abs & p.out_ring_mask;
            for (uint32_t k1 = 0; k1 < kRadix; ++k1) {
                const float re = stage[k2 * kPitch + blk * kRadix + k1] * scale_out;
                const float im = stage[(64u + k2) * kPitch + blk * kRadix + k1] * scale_out;
                out[(uint64_t)(k1 + kRadix * k2) * p.out_ring_blocks + slot] = make_float2(re, im);
            }
        }
        __syncthreads();  // the staging is B1's space again
    }
    if (tid == 0 && *abort_flag) atomicAdd(&g_dft_timeouts, 1u);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
    }
}

template <int P>
int32_t launch(cudaStream_t s, const rv_pfb_fft_params& p, const float2* branch, const float2* tw, float2* out) {
    const void* fn = (const void*)k_dft_tc<P>;
    if (int32_t st = cuda_status(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes),
                                 "dft tc shared memory"))
        return st;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t tiles = (p.block_count + kPair - 1u) / kPair;
    const uint32_t grid = tiles < (uint32_t)sms ? tiles : (uint32_t)sms;
    k_dft_tc<P><<<grid, kThreads, kSmemBytes, s>>>(branch, tw, out, p);
    return cuda_status(cudaGetLastError(), "dft tc");
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace
}  // namespace rv

using namespace rv;

extern "C" int32_t rv_pfb_dft_tc(void* stream, const rv_pfb_fft_params* p, const rv_cf32* branch, uint64_t branch_len,
                                 const rv_cf32* tw, uint64_t tw_len, rv_cf32* ring, uint64_t ring_len, int32_t precision) {
    if (p == nullptr || branch == nullptr || tw == nullptr || ring == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: NULL argument");
    if (p->channels != kM || p->stages != 12)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "pfb dft tc: built for 4096 channels (stages 12), got %u", p->channels);
    if (p->decimation == 0 || kM % p->decimation != 0)
        return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: decimation %u must divide 4096", p->decimation);
    if (!is_pow2(p->out_ring_blocks) || p->out_ring_mask != p->out_ring_blocks - 1u || p->block_count > p->out_ring_blocks)
        return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: out ring of %u blocks (mask %u) for %u blocks",
                             p->out_ring_blocks, p->out_ring_mask, p->block_count);
    if (precision != RV_DFT_FP16 && precision != RV_DFT_BF16)
        return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: precision %d (RV_DFT_FP16 or RV_DFT_BF16)", precision);
    if (tw_len != kM) return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: needs exactly 4096 twiddles");
    if (branch_len < (uint64_t)p->block_count * kM) return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: branch buffer too short");
    if (ring_len < (uint64_t)kM * p->out_ring_blocks) return set_error_fmt(RV_ERR_INVALID, "pfb dft tc: channel ring too short");
    if (p->block_count == 0) return clear_error();
    cudaStream_t s = as_stream(stream);
    const uint32_t zero = 0;
    if (int32_t st = cuda_status(cudaMemcpyToSymbolAsync(g_dft_timeouts, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, s),
                                 "dft tc flag"))
        return st;
    const float2* b = reinterpret_cast<const float2*>(branch);
    const float2* w = reinterpret_cast<const float2*>(tw);
    float2* o = reinterpret_cast<float2*>(ring);
    const int32_t st = precision == RV_DFT_FP16 ? launch<RV_DFT_FP16>(s, *p, b, w, o) : launch<RV_DFT_BF16>(s, *p, b, w, o);
    if (st) return st;
    uint32_t timeouts = 0;
    if (int32_t e = cuda_status(cudaMemcpyFromSymbolAsync(&timeouts, g_dft_timeouts, sizeof timeouts, 0,
                                                          cudaMemcpyDeviceToHost, s),
                                "dft tc flag"))
        return e;
    if (int32_t e = cuda_status(cudaStreamSynchronize(s), "dft tc")) return e;
    if (timeouts) return set_error_fmt(RV_ERR_TIMEOUT, "pfb dft tc: %u CTAs gave up waiting on the tensor cores", timeouts);
    return clear_error();
}
