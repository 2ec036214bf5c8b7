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
// One CTA per SM (225 KB of shared memory), persistent over pairs of blocks.
// A tile's two blocks (64 contiguous KB of branch outputs) arrive through the
// bulk-copy engine (cp.async.bulk, completing on an mbarrier) while the
// previous tile is in the tensor cores. Operands are written to shared memory
// by the threads in the canonical no-swizzle K-major layout (8-row x 16-byte
// core matrices); thread 0 issues the MMAs and commits them to an mbarrier;
// every warp reads its 32 TMEM lanes back with tcgen05.ld, and the Re and Im
// halves of each accumulator meet through a 33 KB exchange. Every mbarrier
// wait is bounded: a wait that runs out sets an error flag the host reads,
// and the CTA lets its copies land, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace rv {
namespace {

constexpr uint32_t kM = 4096;
constexpr uint32_t kRadix = 64;
constexpr uint32_t kPair = 2;                        // blocks per tile
constexpr uint32_t kRows = 128;                      // GEMM M: [Re | Im] x 64
constexpr uint32_t kK = 128;                         // GEMM K: [Re | Im] x 64
constexpr uint32_t kCols = kPair * kRadix;           // GEMM N
constexpr uint32_t kOperand = kRows * kK * 2;        // one 16-bit operand: 32 KB
constexpr uint32_t kBlockBytes = kM * 8;             // one block of branch outputs: 32 KB
constexpr uint32_t kXPitch = kRadix + 1;             // exchange row pitch (odd: no bank conflicts)
constexpr uint32_t kXBytes = kRadix * kXPitch * 4;   // one 64 x 64 FP32 exchange half
constexpr uint32_t kOffA = 0;                        // A_hi, A_lo
constexpr uint32_t kOffB = 2 * kOperand;             // B_hi, B_lo: GEMM 1's operand, then GEMM 2's
constexpr uint32_t kOffRaw = 4 * kOperand;           // the tile's two blocks, prefetched
constexpr uint32_t kOffX = kOffRaw + kPair * kBlockBytes;  // Re and Im exchange halves
constexpr uint32_t kOffMisc = kOffX + 2 * kXBytes;
constexpr uint32_t kSmemBytes = kOffMisc + 128;      // 230,016 bytes
constexpr uint32_t kSplit = 4;                       // threads per accumulator row
constexpr uint32_t kThreads = kRows * kSplit;        // 16 warps
constexpr uint32_t kChunk = kRadix / kSplit;         // columns (or K groups of 8 x 2) per thread
constexpr uint32_t kTmemCols = 256;                  // acc0 at column 0, acc1 at 128
constexpr uint32_t kWaitLimit = 1u << 20;
static_assert(kSmemBytes <= 232448, "shared memory per CTA");
static_assert(kRadix * (kCols + 1) * 4 <= 2 * kXBytes, "the output exchange fits the two halves");

__device__ uint32_t g_dft_timeouts;  // CTAs that stopped on a wait that ran out, since the last status read
__device__ uint32_t g_dft_stop;      // test hook: every CTA stops before it issues a copy or an MMA

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

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// This thread's TMEM row, columns [c0, c0 + 16): acc0 + acc1 2^-s.
template <int P>
__device__ __forceinline__ void combined16(uint32_t tmem, uint32_t c0, float* v) {
    float b[16];
    tmem_ld16(tmem + c0, v);
    tmem_ld16(tmem + kCols + c0, b);
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = v[i] + b[i] * Split<P>::kInvLo;
}

// Rows 0-63 of an accumulator hold Re, rows 64-127 Im, of 64 output indices;
// columns 0-63 belong to the tile's first block, 64-127 to its second. Each
// half of the rows finishes one block: Re rows the first, Im rows the second.
// So each hands the other the part it lacks: Re rows put their second-block
// columns in xa, Im rows their first-block columns in xb. Row `row`'s
// threads split the 64 columns in quarters (q).
template <int P>
__device__ __forceinline__ void exchange(uint32_t lane_tmem, uint32_t row, uint32_t q, float* xa, float* xb) {
    const uint32_t i = row & 63u, other = row < 64u ? kRadix : 0u, c = q * kChunk;
    float* x = row < 64u ? xa : xb;
    float v[16];
    combined16<P>(lane_tmem, other + c, v);
#pragma unroll
    for (int k = 0; k < 16; ++k) x[i * kXPitch + c + (uint32_t)k] = v[k];
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

// The tile's valid blocks (contiguous in the branch buffer) into shared
// memory through the bulk-copy engine, completing on `mbar`.
__device__ __forceinline__ void prefetch(uint32_t raw, const float2* src, uint32_t nblocks, uint32_t mbar) {
    const uint32_t bytes = nblocks * kBlockBytes;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
    for (uint32_t k = 0; k < nblocks; ++k)
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                raw + k * kBlockBytes),
            "l"(src + (uint64_t)k * kM), "r"(kBlockBytes), "r"(mbar)
            : "memory");
}

template <int P>
__global__ void __launch_bounds__(kThreads, 1)
k_dft_tc(const float2* __restrict__ branch, const float2* __restrict__ tw, float2* __restrict__ out,
         rv_pfb_fft_params p) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* const a_hi = sm + kOffA;
    uint8_t* const a_lo = a_hi + kOperand;
    uint8_t* const b_hi = sm + kOffB;
    uint8_t* const b_lo = b_hi + kOperand;
    const float2* const raw = reinterpret_cast<const float2*>(sm + kOffRaw);
    float* const xa = reinterpret_cast<float*>(sm + kOffX);
    float* const xb = xa + kRadix * kXPitch;
    uint64_t* const mbar = reinterpret_cast<uint64_t*>(sm + kOffMisc);  // [0] MMAs, [1] prefetch
    uint32_t* const tmem_slot = reinterpret_cast<uint32_t*>(sm + kOffMisc + 16);
    uint32_t* const abort_flag = reinterpret_cast<uint32_t*>(sm + kOffMisc + 20);
    float* const block_max = reinterpret_cast<float*>(sm + kOffMisc + 32);  // one per warp (16)
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    // thread = (TMEM row, quarter): warp w reads lanes 32 (w % 4) ..; its
    // quarter q = w / 4 takes columns (or K groups) [16 q, 16 q + 16)
    const uint32_t row = tid & (kRows - 1u), q = tid >> 7;
    const uint32_t mbar_mma = smem_addr(mbar), mbar_raw = smem_addr(mbar + 1), raw_addr = smem_addr(raw);
    const uint32_t tiles = (p.block_count + kPair - 1u) / kPair;
    auto valid_in = [&](uint32_t tile) {
        const uint32_t b0 = tile * kPair;
        return p.block_count - b0 < kPair ? p.block_count - b0 : kPair;
    };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_mma));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_raw));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort_flag = *reinterpret_cast<volatile uint32_t*>(&g_dft_stop) != 0u ? 1u : 0u;
    }
    __syncthreads();
    const bool stopped = *abort_flag != 0u;  // read by every thread before any wait can set it
    // thread 0's copies and MMAs in flight: after a stop it waits for them
    // (bounded) before the shared and tensor memory go
    bool raw_pending = false, mma_pending = false;
    uint32_t raw_pending_parity = 0, mma_pending_parity = 0;
    if (tid == 0 && blockIdx.x < tiles && !stopped) {
        prefetch(raw_addr, branch + (uint64_t)blockIdx.x * kPair * kM, valid_in(blockIdx.x), mbar_raw);
        raw_pending = true;
    }
    // A = F in real block form, the same for both stages: row r = [Re | Im]
    // of the output index, column k = [Re | Im] of the summed index.
    {
        const uint32_t kr = row & 63u;
        for (uint32_t j = 4u * q; j < 4u * q + 4u; ++j) {
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint32_t k = 8u * j + (uint32_t)i, kn = k & 63u;
                const float2 f = tw[(kRadix * kr * kn) & (kM - 1u)];
                v[i] = (row < 64u) ? (k < 64u ? f.x : -f.y) : (k < 64u ? f.y : f.x);
            }
            store_split8<P>(a_hi, a_lo, row, 8u * j, v);
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_tmem = tmem + (((warp & 3u) * 32u) << 16);  // this warp's 32 lanes
    const bool re_row = row < 64u;
    const float* const theirs_x = re_row ? xb : xa;

    uint32_t parity_mma = 0, parity_raw = 0;
    for (uint32_t tile = stopped ? tiles : blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t b0 = tile * kPair, nvalid = valid_in(tile);
        const uint32_t blk = row >> 6, i64 = row & 63u, b = b0 + blk;
        const bool valid = blk < nvalid;
        const float2* y = raw + blk * kM;
        const uint32_t m_abs = p.block_base + b;
        const uint32_t dm = ((m_abs & (kM - 1u)) * p.decimation) & (kM - 1u);
        if (wait_parity(mbar_raw, parity_raw)) {
            if (tid == 0) raw_pending = false;
        } else {
            atomicExch(abort_flag, 1u);
        }
        if (tid == 0 && raw_pending) raw_pending_parity = parity_raw;
        parity_raw ^= 1u;
        // the block's largest component, for the power-of-two scale
        float mx = 0.0F;
        if (valid)
            for (uint32_t n1 = kChunk * q; n1 < kChunk * q + kChunk; ++n1) {
                const float2 v = y[(kRadix * n1 + i64 - dm) & (kM - 1u)];
                mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
        if (lane == 0) block_max[warp] = mx;
        __syncthreads();
        if (*abort_flag) break;
        float bmax = 0.0F;  // warps whose lanes are this block's rows: (w % 4) / 2 == blk
#pragma unroll
        for (uint32_t w = 0; w < kThreads / 32u; ++w)
            if (((w & 3u) >> 1) == blk) bmax = fmaxf(bmax, block_max[w]);
        int shift = 0;  // scale = 2^shift puts bmax in [2^13, 2^14)
        if (bmax > 0.0F) {
            const int e = (int)((__float_as_uint(bmax) >> 23) & 0xFFu) - 127;
            shift = 13 - e;
            shift = shift > 100 ? 100 : (shift < -100 ? -100 : shift);
        }
        const float scale_in = ldexpf(1.0F, shift);
        // B1 row (blk, n2 = i64): K = [Re | Im] of y'[64 n1 + n2]; this
        // quarter's n1 = 16 q .. 16 q + 15
        for (uint32_t j = 2u * q; j < 2u * q + 2u; ++j) {
            float re[8], im[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint32_t n1 = 8u * j + (uint32_t)k;
                const float2 v = valid ? y[(kRadix * n1 + i64 - dm) & (kM - 1u)] : make_float2(0.0F, 0.0F);
                re[k] = v.x * scale_in;
                im[k] = v.y * scale_in;
            }
            store_split8<P>(b_hi, b_lo, row, 8u * j, re);
            store_split8<P>(b_hi, b_lo, row, kRadix + 8u * j, im);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            issue_gemm<P>(tmem, smem_addr(a_hi), smem_addr(a_lo), smem_addr(b_hi), smem_addr(b_lo), mbar_mma);
            mma_pending = true, mma_pending_parity = parity_mma;
            const uint32_t next = tile + gridDim.x;  // the raw blocks are read: fetch the next tile's
            if (next < tiles && !raw_pending) {
                fence_async_smem();
                prefetch(raw_addr, branch + (uint64_t)next * kPair * kM, valid_in(next), mbar_raw);
                raw_pending = true, raw_pending_parity = parity_raw;
            }
        }
        if (wait_parity(mbar_mma, parity_mma)) {
            if (tid == 0) mma_pending = false;
        } else {
            atomicExch(abort_flag, 1u);
        }
        parity_mma ^= 1u;
        __syncthreads();
        if (*abort_flag) break;
        fence_after();
        // GEMM 1 out, times 2^-6: Re Z[k1] in rows k1, Im in 64 + k1
        exchange<P>(lane_tmem, row, q, xa, xb);
        __syncthreads();
        // B2 row (blk, k1 = i64): K = [Re | Im] of Z'[k1][n2] = Z[k1][n2] W^(k1 n2)
        {
            const uint32_t c = kChunk * q;
            float own[16];
            combined16<P>(lane_tmem, blk * kRadix + c, own);
#pragma unroll
            for (uint32_t j = 0; j < 16; j += 8) {
                float2 w[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) w[k] = tw[(i64 * (c + j + (uint32_t)k)) & (kM - 1u)];
                float re[8], im[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const uint32_t n2 = c + j + (uint32_t)k;
                    const float mine = own[j + (uint32_t)k] * (1.0F / 64.0F);
                    const float theirs = theirs_x[i64 * kXPitch + n2] * (1.0F / 64.0F);
                    const float zr = re_row ? mine : theirs, zi = re_row ? theirs : mine;
                    re[k] = zr * w[k].x - zi * w[k].y;
                    im[k] = zr * w[k].y + zi * w[k].x;
                }
                store_split8<P>(b_hi, b_lo, row, c + j, re);
                store_split8<P>(b_hi, b_lo, row, kRadix + c + j, im);
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            issue_gemm<P>(tmem, smem_addr(a_hi), smem_addr(a_lo), smem_addr(b_hi), smem_addr(b_lo), mbar_mma);
            mma_pending = true, mma_pending_parity = parity_mma;
        }
        if (wait_parity(mbar_mma, parity_mma)) {
            if (tid == 0) mma_pending = false;
        } else {
            atomicExch(abort_flag, 1u);
        }
        parity_mma ^= 1u;
        __syncthreads();
        if (*abort_flag) break;
        fence_after();
        // GEMM 2 out: Re Y[k1 + 64 k2] in rows k2, Im in 64 + k2, columns
        // (block, k1). The Im rows hand over both blocks' columns; the Re
        // rows then write each channel's two adjacent ring slots together.
        {
            const uint32_t c = kChunk * q;
            float own0[16], own1[16];
            combined16<P>(lane_tmem, c, own0);
            combined16<P>(lane_tmem, kRadix + c, own1);
            float* const x2 = xa;  // [64][kCols + 1]: both halves of the exchange
            if (!re_row) {
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    x2[i64 * (kCols + 1u) + c + (uint32_t)k] = own0[k];
                    x2[i64 * (kCols + 1u) + kRadix + c + (uint32_t)k] = own1[k];
                }
            }
            __syncthreads();
            if (re_row) {
                // times 2^6 2^-shift undoes both scales, per block
                float s_out[kPair];
#pragma unroll
                for (uint32_t bb = 0; bb < kPair; ++bb) {
                    float bm = 0.0F;
#pragma unroll
                    for (uint32_t w = 0; w < kThreads / 32u; ++w)
                        if (((w & 3u) >> 1) == bb) bm = fmaxf(bm, block_max[w]);
                    int sh = 0;
                    if (bm > 0.0F) {
                        sh = 13 - ((int)((__float_as_uint(bm) >> 23) & 0xFFu) - 127);
                        sh = sh > 100 ? 100 : (sh < -100 ? -100 : sh);
                    }
                    s_out[bb] = ldexpf(64.0F, -sh);
                }
                const uint32_t slot0 = (p.block_base + b0) & p.out_ring_mask;
                const uint32_t slot1 = (p.block_base + b0 + 1u) & p.out_ring_mask;
                const bool pair = nvalid == kPair && slot1 == slot0 + 1u && (slot0 & 1u) == 0u &&
                                  (reinterpret_cast<uintptr_t>(out) & 15u) == 0u;
#pragma unroll
                for (uint32_t k = 0; k < 16; ++k) {
                    const uint32_t k1 = c + k;
                    const float r0 = own0[k] * s_out[0], i0 = x2[i64 * (kCols + 1u) + k1] * s_out[0];
                    const float r1 = own1[k] * s_out[1], i1 = x2[i64 * (kCols + 1u) + kRadix + k1] * s_out[1];
                    float2* const dst = out + (uint64_t)(k1 + kRadix * i64) * p.out_ring_blocks;
                    if (pair) {
                        *reinterpret_cast<float4*>(dst + slot0) = make_float4(r0, i0, r1, i1);
                    } else {
                        dst[slot0] = make_float2(r0, i0);
                        if (nvalid == kPair) dst[slot1] = make_float2(r1, i1);
                    }
                }
            }
        }
        fence_before();
        __syncthreads();  // B and the exchange are free for the next tile
    }
    // after a stop, a prefetch or MMAs still in flight finish (bounded)
    // before the CTA frees its tensor memory and leaves
    if (tid == 0 && raw_pending) wait_parity(mbar_raw, raw_pending_parity);
    if (tid == 0 && mma_pending) wait_parity(mbar_mma, mma_pending_parity);
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
    const float2* b = reinterpret_cast<const float2*>(branch);
    const float2* w = reinterpret_cast<const float2*>(tw);
    float2* o = reinterpret_cast<float2*>(ring);
    const int32_t st = precision == RV_DFT_FP16 ? launch<RV_DFT_FP16>(s, *p, b, w, o) : launch<RV_DFT_BF16>(s, *p, b, w, o);
    if (st) return st;
    return clear_error();
}

extern "C" int32_t rv_pfb_dft_tc_status(void* stream, uint32_t* timeouts) {
    cudaStream_t s = as_stream(stream);
    uint32_t count = 0;
    const uint32_t zero = 0;
    if (int32_t e = cuda_status(cudaMemcpyFromSymbolAsync(&count, g_dft_timeouts, sizeof count, 0, cudaMemcpyDeviceToHost, s),
                                "dft tc status"))
        return e;
    if (int32_t e = cuda_status(cudaMemcpyToSymbolAsync(g_dft_timeouts, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, s),
                                "dft tc status"))
        return e;
    if (int32_t e = cuda_status(cudaStreamSynchronize(s), "dft tc status")) return e;
    if (timeouts) *timeouts = count;
    if (count) return set_error_fmt(RV_ERR_TIMEOUT, "pfb dft tc: %u CTAs gave up waiting on the tensor cores", count);
    return clear_error();
}

extern "C" int32_t rv_pfb_dft_tc_stop_for_test(void* stream, int32_t stop) {
    const uint32_t v = stop ? 1u : 0u;
    return cuda_status(cudaMemcpyToSymbolAsync(g_dft_stop, &v, sizeof v, 0, cudaMemcpyHostToDevice, as_stream(stream)),
                       "dft tc stop");
}
