// The learned detection proposal's network: a small spectrogram CNN whose
// forward and backward passes run as BF16 GEMMs on the tcgen05 tensor cores
// with FP32 accumulators in tensor memory.
//
// Every convolution is an implicit GEMM. One kernel, k_gemm, computes
//   D[m][n] (op)= sum_k A(m, k) B(n, k)
// where A and B are read through "operand" descriptors: a strided matrix, the
// im2col patch matrix of an NHWC activation (row = output pixel, column =
// (kh, kw, c)), or that patch matrix transposed. The threads gather a 128-row
// by 64-column chunk of each operand, round it to BF16 and store it in shared
// memory in the canonical no-swizzle K-major layout; thread 0 issues four
// tcgen05.mma (K = 16 each) per chunk and commits them to an mbarrier while the
// threads gather the next chunk into the other buffer. The epilogue reads the
// accumulator back with tcgen05.ld and stores (optionally with bias and ReLU),
// atomically adds (split-K weight gradients), or scatters it back through the
// patch geometry (col2im: input gradients).
//
//   forward, layer l:  Y_l = act(patch(X_{l-1}) W_l^T + b_l)
//   backward:          dZ_l = dY_l * [Y_l > 0]
//                      dW_l = dZ_l^T patch(X_{l-1})          (split over pixels)
//                      db_l = column sums of dZ_l
//                      dX_{l-1} = col2im(dZ_l W_l)
//
// The network (input tiles of 64 frames x 256 bins x 2 channels, BF16, NHWC):
//   conv1 4x4 stride 4x4,           2 -> 64, ReLU   -> 16 x 64 x 64
//   conv2 2x2 stride 2x2,          64 -> 128, ReLU  ->  8 x 32 x 128
//   conv3 2x3 stride 2x1 pad 0x1, 128 -> 128, ReLU  ->  4 x 32 x 128
//   conv4 4x3 stride 4x1 pad 0x1, 128 -> 64, ReLU   ->  1 x 32 x 64
//   head  1x1,                     64 -> 1          ->  1 x 32 logits
// 231,873 parameters; one logit per 8-bin cell of the tile.
//
// Every mbarrier wait is bounded; a wait that runs out counts in the
// network's device status word and the CTA waits (bounded) for the MMAs it
// committed before it frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <random>
#include <vector>

#include "common.cuh"
#include "tc.cuh"

namespace rv {
namespace {

constexpr uint32_t kRows = 128;      // MMA M: output rows per CTA
constexpr uint32_t kKc = 64;         // K elements per staged chunk (four MMAs)
constexpr uint32_t kThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kOperandA = kRows * kKc * 2;  // 16 KB

enum : uint32_t { kMatrix = 0, kPatch = 1, kPatchT = 2 };
enum : uint32_t { kStore = 0, kBiasRelu = 1, kBias = 2, kAtomic = 3, kCol2im = 4 };

// NHWC input geometry of a patch operand and the convolution over it.
struct Conv {
    uint32_t h, w, c;
    uint32_t kh, kw, sh, sw, ph, pw;
    uint32_t ho, wo;
};

struct Operand {
    const void* base;
    uint32_t kind;   // kMatrix, kPatch, kPatchT
    uint32_t bf16;   // element type: 0 FP32, 1 BF16
    uint32_t rows;   // rows of this operand (A: m, B: n); rows at or past it read zero
    uint32_t pad;
    uint64_t rs, ks; // kMatrix element strides of a row and of k
    Conv g;
};

struct GemmArgs {
    Operand a, b;
    uint32_t m, n, k;
    uint32_t k_split;  // K elements per CTA along grid z (a multiple of kKc)
    float* d;
    uint64_t ldd;
    uint32_t epilogue;
    uint32_t pad;
    const float* bias;
    Conv out;          // kCol2im: the geometry D's (pixel, patch column) scatter through
    uint32_t* status;
};

__device__ __forceinline__ float load_one(const Operand& o, uint64_t idx) {
    if (o.bf16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(o.base)[idx]);
    return reinterpret_cast<const float*>(o.base)[idx];
}

// Element index of patch entry (pixel, column) of geometry g, or -1 in the
// zero padding.
__device__ __forceinline__ int64_t patch_index(const Conv& g, uint32_t pixel, uint32_t col) {
    const uint32_t per_image = g.ho * g.wo;
    const uint32_t img = pixel / per_image, rem = pixel - img * per_image;
    const uint32_t oh = rem / g.wo, ow = rem - oh * g.wo;
    const uint32_t kwc = g.kw * g.c;
    const uint32_t kh = col / kwc, r2 = col - kh * kwc;
    const uint32_t kw = r2 / g.c, c = r2 - kw * g.c;
    const int32_t h = (int32_t)(oh * g.sh + kh) - (int32_t)g.ph;
    const int32_t w = (int32_t)(ow * g.sw + kw) - (int32_t)g.pw;
    if (h < 0 || w < 0 || h >= (int32_t)g.h || w >= (int32_t)g.w) return -1;
    return (((int64_t)img * g.h + h) * g.w + w) * g.c + c;
}

// Eight consecutive K entries (k0 .. k0 + 7) of operand row r; zero past the
// operand's rows or K.
__device__ __forceinline__ void gather8(const Operand& o, uint32_t r, uint32_t k0, uint32_t kmax, float* v) {
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = 0.0F;
    if (r >= o.rows || k0 >= kmax) return;
    const bool full = k0 + 8u <= kmax;
    if (o.kind == kMatrix) {
        const uint64_t base = (uint64_t)r * o.rs + (uint64_t)k0 * o.ks;
        if (full && o.ks == 1 && !o.bf16 && (base & 3u) == 0 &&
            (reinterpret_cast<uintptr_t>(o.base) & 15u) == 0) {
            const float4* p = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(o.base) + base);
            const float4 x = p[0], y = p[1];
            v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w, v[4] = y.x, v[5] = y.y, v[6] = y.z, v[7] = y.w;
            return;
        }
        for (uint32_t i = 0; i < 8u && k0 + i < kmax; ++i) v[i] = load_one(o, base + (uint64_t)i * o.ks);
        return;
    }
    if (o.kind == kPatch) {
        // channels contiguous: eight columns share (kh, kw) when C % 8 == 0,
        // or one (kh) row of the patch when KW * C == 8 and there is no
        // horizontal padding
        if (full && ((o.g.c & 7u) == 0 || (o.g.kw * o.g.c == 8u && o.g.pw == 0))) {
            const int64_t idx = patch_index(o.g, r, k0);
            if (idx < 0) return;  // the whole run lies in the padding
            if (!o.bf16 && (idx & 3) == 0 && (reinterpret_cast<uintptr_t>(o.base) & 15u) == 0) {
                const float4* p = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(o.base) + idx);
                const float4 x = p[0], y = p[1];
                v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w, v[4] = y.x, v[5] = y.y, v[6] = y.z, v[7] = y.w;
                return;
            }
            if (o.bf16 && (idx & 7) == 0 && (reinterpret_cast<uintptr_t>(o.base) & 15u) == 0) {
                const uint4 q = *reinterpret_cast<const uint4*>(reinterpret_cast<const __nv_bfloat16*>(o.base) + idx);
                const uint32_t words[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    v[2 * i] = __uint_as_float(words[i] << 16);
                    v[2 * i + 1] = __uint_as_float(words[i] & 0xFFFF0000u);
                }
                return;
            }
            for (uint32_t i = 0; i < 8u; ++i) v[i] = load_one(o, (uint64_t)idx + i);
            return;
        }
        for (uint32_t i = 0; i < 8u && k0 + i < kmax; ++i) {
            const int64_t idx = patch_index(o.g, r, k0 + i);
            if (idx >= 0) v[i] = load_one(o, (uint64_t)idx);
        }
        return;
    }
    // kPatchT: row r is the patch column, K runs over pixels
    for (uint32_t i = 0; i < 8u && k0 + i < kmax; ++i) {
        const int64_t idx = patch_index(o.g, k0 + i, r);
        if (idx >= 0) v[i] = load_one(o, (uint64_t)idx);
    }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Rows [0, rows) x K chunk [k0, k0 + kKc) of an operand into shared memory.
__device__ __forceinline__ void stage(const Operand& o, uint32_t row0, uint32_t rows, uint32_t k0, uint32_t kmax,
                                     uint8_t* dst) {
    for (uint32_t e = threadIdx.x; e < rows * (kKc / 8u); e += kThreads) {
        const uint32_t r = e >> 3, g = e & 7u;
        float v[8];
        gather8(o, row0 + r, k0 + 8u * g, kmax, v);
        const uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                                   pack_bf16(v[6], v[7]));
        *reinterpret_cast<uint4*>(dst + tc::core_offset(r, 8u * g, kKc)) = q;
    }
}

template <uint32_t NT>
__global__ void __launch_bounds__(kThreads) k_gemm(const GemmArgs g) {
    constexpr uint32_t kOperandB = NT * kKc * 2;
    constexpr uint32_t kStage = kOperandA + kOperandB;
    constexpr uint32_t kCols = NT < 32u ? 32u : NT;
    constexpr uint32_t idesc = tc::instr_desc_f16(1u, kRows, NT);
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* const mbar = reinterpret_cast<uint64_t*>(sm + 2 * kStage);
    uint32_t* const slot = reinterpret_cast<uint32_t*>(sm + 2 * kStage + 16);
    uint32_t* const abort_flag = slot + 1;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t m0 = blockIdx.x * kRows, n0 = blockIdx.y * NT;
    const uint32_t kbeg = blockIdx.z * g.k_split;
    const uint32_t kend = min(g.k, kbeg + g.k_split);
    const uint32_t chunks = kend > kbeg ? (kend - kbeg + kKc - 1u) / kKc : 0u;

    if (warp == 0) tc::tmem_alloc(tc::smem_addr(slot), kCols);
    if (tid == 0) {
        tc::mbar_init(tc::smem_addr(mbar), 1);
        tc::mbar_init(tc::smem_addr(mbar + 1), 1);
        tc::mbar_fence_init();
        *abort_flag = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *slot;

    Operand a = g.a, b = g.b;
    uint32_t issued = 0;
    for (uint32_t c = 0; c < chunks; ++c) {
        const uint32_t buf = c & 1u;
        if (c >= 2u && tid == 0)
            if (!tc::wait_parity(tc::smem_addr(mbar + buf), ((c >> 1) + 1u) & 1u, kWaitLimit)) *abort_flag = 1u;
        __syncthreads();
        if (*abort_flag) break;
        uint8_t* const sa = sm + buf * kStage;
        uint8_t* const sb = sa + kOperandA;
        const uint32_t k0 = kbeg + c * kKc;
        stage(a, m0, kRows, k0, kend, sa);
        stage(b, n0, NT, k0, kend, sb);
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint32_t a_addr = tc::smem_addr(sa), b_addr = tc::smem_addr(sb);
#pragma unroll
            for (uint32_t s = 0; s < kKc / 16u; ++s)
                tc::mma_f16(tmem, tc::smem_desc(a_addr + 256u * s, kKc * 16u), tc::smem_desc(b_addr + 256u * s, kKc * 16u),
                            idesc, (c > 0u || s > 0u) ? 1u : 0u);
            tc::commit(tc::smem_addr(mbar + buf));
        }
        issued = c + 1u;
    }
    // the last commit covers every MMA issued before it
    if (tid == 0 && issued > 0u) {
        const uint32_t last = issued - 1u;
        if (!tc::wait_parity(tc::smem_addr(mbar + (last & 1u)), (last >> 1) & 1u, kWaitLimit)) {
            *abort_flag = 1u;
            tc::wait_parity(tc::smem_addr(mbar + (last & 1u)), (last >> 1) & 1u, kWaitLimit);
        }
    }
    __syncthreads();
    tc::fence_after();
    if (!*abort_flag) {
        const uint32_t row = warp * 32u + lane, m = m0 + row;
        const uint32_t lane_tmem = tmem + ((warp * 32u) << 16);
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < NT; c0 += 16u) {
            float v[16];
            if (issued > 0u) {
                tc::tmem_ld16(lane_tmem + c0, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.0F;
            }
            if (m >= g.m) continue;
#pragma unroll
            for (uint32_t j = 0; j < 16u; ++j) {
                const uint32_t n = n0 + c0 + j;
                if (n >= g.n) break;
                float x = v[j];
                switch (g.epilogue) {
                    case kStore:
                        g.d[(uint64_t)m * g.ldd + n] = x;
                        break;
                    case kBiasRelu:
                        x = x + g.bias[n];
                        g.d[(uint64_t)m * g.ldd + n] = x > 0.0F ? x : 0.0F;
                        break;
                    case kBias:
                        g.d[(uint64_t)m * g.ldd + n] = x + g.bias[n];
                        break;
                    case kAtomic:
                        atomicAdd(&g.d[(uint64_t)m * g.ldd + n], x);
                        break;
                    default: {  // kCol2im
                        const int64_t idx = patch_index(g.out, m, n);
                        if (idx >= 0) atomicAdd(&g.d[idx], x);
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicAdd(g.status, 1u);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, kCols);
    }
}

// ---- the forward pass's GEMM: BF16 operands copied by cp.async ----------
//
// A is the patch matrix of a BF16 NHWC activation whose eight-column runs are
// contiguous (C % 8 == 0, or one kernel row when KW * C == 8 without
// horizontal padding); B is a BF16 [N][K] weight matrix (K % 8 == 0). Every
// 16-byte run goes global -> shared by cp.async (zero-filled in the padding
// and past the edges), kFwdStages chunks in flight, so the gathers overlap
// one another and the tensor cores. Epilogue: bias, then ReLU to BF16 or the
// plain FP32 result.
constexpr uint32_t kFwdStages = 3;

struct FwdArgs {
    const __nv_bfloat16* x;  // activation (NHWC)
    const __nv_bfloat16* w;  // [n][k]
    const float* bias;
    Conv g;
    uint32_t m, n, k;
    uint32_t relu;           // 1: ReLU, BF16 out; 0: FP32 out
    void* d;                 // [m][n]
    uint32_t* status;
};

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <uint32_t NT>
__global__ void __launch_bounds__(kThreads) k_gemm_fwd(const FwdArgs f) {
    constexpr uint32_t kOperandB = NT * kKc * 2;
    constexpr uint32_t kStage = kOperandA + kOperandB;
    constexpr uint32_t kCols = NT < 32u ? 32u : NT;
    constexpr uint32_t idesc = tc::instr_desc_f16(1u, kRows, NT);
    constexpr uint32_t kRowsPer = kRows / 16u;  // A rows per thread (8 threads share a row's groups)
    constexpr uint32_t kBRowsPer = NT >= 16u ? NT / 16u : 1u;
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* const mbar = reinterpret_cast<uint64_t*>(sm + kFwdStages * kStage);
    uint32_t* const slot = reinterpret_cast<uint32_t*>(sm + kFwdStages * kStage + 8 * kFwdStages);
    uint32_t* const abort_flag = slot + 1;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t m0 = blockIdx.x * kRows, n0 = blockIdx.y * NT;
    const uint32_t chunks = (f.k + kKc - 1u) / kKc;
    const uint32_t g8 = (tid & 7u) * 8u;  // this thread's column run within a chunk
    const uint32_t rsub = tid >> 3;       // rows rsub + 16 j

    if (warp == 0) tc::tmem_alloc(tc::smem_addr(slot), kCols);
    if (tid == 0) {
        for (uint32_t b = 0; b < kFwdStages; ++b) tc::mbar_init(tc::smem_addr(mbar + b), 1);
        tc::mbar_fence_init();
        *abort_flag = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *slot;

    // per A row: the image's element offset and the patch origin, or invalid
    const uint32_t per_image = f.g.ho * f.g.wo;
    int64_t row_base[kRowsPer];
    int32_t row_h[kRowsPer], row_w[kRowsPer];
#pragma unroll
    for (uint32_t j = 0; j < kRowsPer; ++j) {
        const uint32_t m = m0 + rsub + 16u * j;
        if (m < f.m) {
            const uint32_t img = m / per_image, rem = m - img * per_image;
            const uint32_t oh = rem / f.g.wo, ow = rem - oh * f.g.wo;
            row_base[j] = (int64_t)img * f.g.h * f.g.w * f.g.c;
            row_h[j] = (int32_t)(oh * f.g.sh) - (int32_t)f.g.ph;
            row_w[j] = (int32_t)(ow * f.g.sw) - (int32_t)f.g.pw;
        } else {
            row_base[j] = -1;
            row_h[j] = row_w[j] = 0;
        }
    }
    const uint32_t kwc = f.g.kw * f.g.c;

    auto issue = [&](uint32_t c) {
        uint8_t* const sa = sm + (c % kFwdStages) * kStage;
        uint8_t* const sb = sa + kOperandA;
        const uint32_t k = c * kKc + g8;
        const bool k_ok = k < f.k;
        const uint32_t kh = k_ok ? k / kwc : 0u, r2 = k_ok ? k - kh * kwc : 0u;
        const uint32_t kw = r2 / f.g.c, ch = r2 - kw * f.g.c;
#pragma unroll
        for (uint32_t j = 0; j < kRowsPer; ++j) {
            const uint32_t r = rsub + 16u * j;
            const int32_t h = row_h[j] + (int32_t)kh, w = row_w[j] + (int32_t)kw;
            const bool ok = k_ok && row_base[j] >= 0 && h >= 0 && w >= 0 && h < (int32_t)f.g.h && w < (int32_t)f.g.w;
            const __nv_bfloat16* src =
                ok ? f.x + row_base[j] + ((int64_t)h * f.g.w + w) * f.g.c + ch : f.x;
            cp_async16(tc::smem_addr(sa + tc::core_offset(r, g8, kKc)), src, ok ? 16u : 0u);
        }
#pragma unroll
        for (uint32_t j = 0; j < kBRowsPer; ++j) {
            const uint32_t r = rsub + 16u * j;
            if (r >= NT) break;
            const uint32_t nrow = n0 + r;
            const bool ok = k_ok && nrow < f.n;
            const __nv_bfloat16* src = ok ? f.w + (uint64_t)nrow * f.k + k : f.w;
            cp_async16(tc::smem_addr(sb + tc::core_offset(r, g8, kKc)), src, ok ? 16u : 0u);
        }
    };

#pragma unroll
    for (uint32_t c = 0; c + 1u < kFwdStages; ++c) {
        if (c < chunks) issue(c);
        cp_async_commit();
    }
    uint32_t issued = 0;
    for (uint32_t c = 0; c < chunks; ++c) {
        cp_async_wait<kFwdStages - 2>();
        tc::fence_async_smem();
        __syncthreads();
        if (*abort_flag) break;
        if (tid == 0) {
            tc::fence_after();
            uint8_t* const sa = sm + (c % kFwdStages) * kStage;
            const uint32_t a_addr = tc::smem_addr(sa), b_addr = a_addr + kOperandA;
#pragma unroll
            for (uint32_t s = 0; s < kKc / 16u; ++s)
                tc::mma_f16(tmem, tc::smem_desc(a_addr + 256u * s, kKc * 16u),
                            tc::smem_desc(b_addr + 256u * s, kKc * 16u), idesc, (c > 0u || s > 0u) ? 1u : 0u);
            tc::commit(tc::smem_addr(mbar + (c % kFwdStages)));
        }
        issued = c + 1u;
        const uint32_t next = c + kFwdStages - 1u;  // into the stage chunk c - 1 used
        if (next < chunks) {
            if (c >= 1u) {
                if (tid == 0 && !tc::wait_parity(tc::smem_addr(mbar + ((c - 1u) % kFwdStages)),
                                                 ((c - 1u) / kFwdStages) & 1u, kWaitLimit))
                    *abort_flag = 1u;
                __syncthreads();
                if (*abort_flag) {
                    cp_async_commit();
                    break;
                }
            }
            issue(next);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (tid == 0 && issued > 0u) {
        const uint32_t last = issued - 1u;
        const uint32_t bar = tc::smem_addr(mbar + (last % kFwdStages)), par = (last / kFwdStages) & 1u;
        if (!tc::wait_parity(bar, par, kWaitLimit)) {
            *abort_flag = 1u;
            tc::wait_parity(bar, par, kWaitLimit);
        }
    }
    __syncthreads();
    tc::fence_after();
    if (!*abort_flag && issued == chunks) {
        const uint32_t row = warp * 32u + lane, m = m0 + row;
        const uint32_t lane_tmem = tmem + ((warp * 32u) << 16);
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < NT; c0 += 16u) {
            float v[16];
            tc::tmem_ld16(lane_tmem + c0, v);
            if (m >= f.m) continue;
            const uint32_t nb = n0 + c0;
            if (f.relu) {
                __nv_bfloat16* const out = reinterpret_cast<__nv_bfloat16*>(f.d) + (uint64_t)m * f.n + nb;
                if (nb + 16u <= f.n && (f.n & 7u) == 0) {
                    uint32_t q[8];
#pragma unroll
                    for (uint32_t j = 0; j < 8u; ++j) {
                        const float a = fmaxf(v[2 * j] + f.bias[nb + 2 * j], 0.0F);
                        const float b = fmaxf(v[2 * j + 1] + f.bias[nb + 2 * j + 1], 0.0F);
                        q[j] = pack_bf16(a, b);
                    }
                    reinterpret_cast<uint4*>(out)[0] = make_uint4(q[0], q[1], q[2], q[3]);
                    reinterpret_cast<uint4*>(out)[1] = make_uint4(q[4], q[5], q[6], q[7]);
                } else {
                    for (uint32_t j = 0; j < 16u && nb + j < f.n; ++j)
                        out[j] = __float2bfloat16_rn(fmaxf(v[j] + f.bias[nb + j], 0.0F));
                }
            } else {
                float* const out = reinterpret_cast<float*>(f.d) + (uint64_t)m * f.n + nb;
                for (uint32_t j = 0; j < 16u && nb + j < f.n; ++j) out[j] = v[j] + f.bias[nb + j];
            }
        }
    } else if (tid == 0 && *abort_flag) {
        atomicAdd(f.status, 1u);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, kCols);
    }
}

template <uint32_t NT>
constexpr uint32_t fwd_smem() {
    return kFwdStages * (kOperandA + NT * kKc * 2u) + 64u;
}

template <uint32_t NT>
int32_t launch_fwd(cudaStream_t s, const FwdArgs& f) {
    if (int32_t st = ensure_shared((const void*)k_gemm_fwd<NT>, fwd_smem<NT>(), "cnn forward shared memory"))
        return st;
    const dim3 grid((f.m + kRows - 1u) / kRows, (f.n + NT - 1u) / NT, 1);
    k_gemm_fwd<NT><<<grid, kThreads, fwd_smem<NT>(), s>>>(f);
    return cuda_status(cudaGetLastError(), "cnn forward gemm");
}

int32_t gemm_fwd(cudaStream_t s, const FwdArgs& f) {
    if (f.m == 0 || f.n == 0) return RV_OK;
    if (f.k % 8u != 0 || !((f.g.c % 8u) == 0 || (f.g.kw * f.g.c == 8u && f.g.pw == 0)) ||
        (reinterpret_cast<uintptr_t>(f.x) & 15u) != 0 || (reinterpret_cast<uintptr_t>(f.w) & 15u) != 0)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "cnn forward: operands without contiguous 16-byte runs");
    if (f.n <= 16u) return launch_fwd<16>(s, f);
    if (f.n <= 32u) return launch_fwd<32>(s, f);
    if (f.n <= 64u) return launch_fwd<64>(s, f);
    return launch_fwd<128>(s, f);
}

template <uint32_t NT>
constexpr uint32_t gemm_smem() {
    return 2u * (kOperandA + NT * kKc * 2u) + 64u;
}

template <uint32_t NT>
int32_t launch_gemm(cudaStream_t s, const GemmArgs& g, uint32_t splits) {
    if (int32_t st = ensure_shared((const void*)k_gemm<NT>, gemm_smem<NT>(), "cnn gemm shared memory")) return st;
    const dim3 grid((g.m + kRows - 1u) / kRows, (g.n + NT - 1u) / NT, splits);
    k_gemm<NT><<<grid, kThreads, gemm_smem<NT>(), s>>>(g);
    return cuda_status(cudaGetLastError(), "cnn gemm");
}

// Picks the column tile and, for atomically accumulated results, the K split
// that gives the GPU about two waves of CTAs.
int32_t gemm(cudaStream_t s, GemmArgs g, int sms) {
    if (g.m == 0 || g.n == 0) return RV_OK;
    uint32_t nt = g.n <= 16u ? 16u : g.n <= 32u ? 32u : g.n <= 64u ? 64u : 128u;
    const uint64_t tiles = (uint64_t)((g.m + kRows - 1u) / kRows) * ((g.n + nt - 1u) / nt);
    uint32_t splits = 1;
    if (g.epilogue == kAtomic) {
        const uint64_t want = 2ull * (uint64_t)sms;
        const uint32_t chunks = (g.k + kKc - 1u) / kKc;
        if (tiles < want) splits = (uint32_t)std::min<uint64_t>(chunks, (want + tiles - 1u) / tiles);
        splits = std::max(splits, 1u);
    }
    const uint32_t chunks_per = ((g.k + kKc - 1u) / kKc + splits - 1u) / splits;
    g.k_split = chunks_per * kKc;
    splits = (g.k + g.k_split - 1u) / g.k_split;
    switch (nt) {
        case 16: return launch_gemm<16>(s, g, splits);
        case 32: return launch_gemm<32>(s, g, splits);
        case 64: return launch_gemm<64>(s, g, splits);
        default: return launch_gemm<128>(s, g, splits);
    }
}

// ---- elementwise kernels ----------------------------------------------

__global__ void k_relu_grad(float* __restrict__ dy, const __nv_bfloat16* __restrict__ y, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[i]) > 0.0F)) dy[i] = 0.0F;
}

// The BF16 copy of the weights the forward pass reads (biases stay FP32).
__global__ void k_to_bf16(const float* __restrict__ p, uint64_t n, __nv_bfloat16* __restrict__ q) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        q[i] = __float2bfloat16_rn(p[i]);
}

// db[c] += sum over rows of dz[row][c]; a block per 32-column group, rows
// split over the grid's y dimension.
__global__ void k_bias_grad(const float* __restrict__ dz, uint32_t rows, uint32_t cols, float* __restrict__ db) {
    const uint32_t c = blockIdx.x * 32u + (threadIdx.x & 31u);
    const uint32_t r_lane = threadIdx.x >> 5, r_lanes = blockDim.x >> 5;
    float acc = 0.0F;
    if (c < cols)
        for (uint32_t r = blockIdx.y * r_lanes + r_lane; r < rows; r += gridDim.y * r_lanes) acc += dz[(uint64_t)r * cols + c];
    __shared__ float part[32][33];
    part[r_lane][threadIdx.x & 31u] = acc;
    __syncthreads();
    if (r_lane == 0 && c < cols) {
        float t = 0.0F;
        for (uint32_t i = 0; i < r_lanes; ++i) t += part[i][threadIdx.x & 31u];
        atomicAdd(&db[c], t);
    }
}

// Weighted binary cross-entropy with logits, mean over n: loss and dlogits.
__global__ void k_bce(const float* __restrict__ z, const float* __restrict__ y, uint32_t n, float pos_weight,
                      float* __restrict__ dz, float* __restrict__ loss) {
    float acc = 0.0F;
    const float inv = 1.0F / (float)n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = z[i], t = y[i];
        // log(1 + e^-|x|) + max(-x, 0) = -log sigmoid(x); the same for -x
        const float soft = log1pf(expf(-fabsf(x)));
        const float nl_pos = soft + fmaxf(-x, 0.0F), nl_neg = soft + fmaxf(x, 0.0F);
        acc += pos_weight * t * nl_pos + (1.0F - t) * nl_neg;
        const float s = 1.0F / (1.0F + expf(-x));
        dz[i] = (s * (pos_weight * t + 1.0F - t) - pos_weight * t) * inv;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    if ((threadIdx.x & 31u) == 0) atomicAdd(loss, acc * inv);
}

struct AdamArgs {
    float lr, beta1, beta2, eps, c1, c2, weight_decay;
};

// One Adam step; also refreshes the BF16 copy the forward pass reads.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       uint64_t n, AdamArgs a, __nv_bfloat16* __restrict__ q) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float gi = g[i] + a.weight_decay * p[i];
        const float mi = a.beta1 * m[i] + (1.0F - a.beta1) * gi;
        const float vi = a.beta2 * v[i] + (1.0F - a.beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - a.lr * (mi / a.c1) / (sqrtf(vi / a.c2) + a.eps);
        p[i] = pi;
        q[i] = __float2bfloat16_rn(pi);
    }
}

// ---- the network ------------------------------------------------------

struct Layer {
    Conv g;            // geometry over the layer's input
    uint32_t cout;
    uint32_t relu;
    uint64_t w_off, b_off;  // into the parameter vector
    uint32_t k() const { return g.kh * g.kw * g.c; }
    uint64_t pixels() const { return (uint64_t)g.ho * g.wo; }
};

constexpr uint32_t kLayers = 5;

void describe(Layer* L) {
    // input 64 x 256 x 2
    L[0] = Layer{{64, 256, 2, 4, 4, 4, 4, 0, 0, 16, 64}, 64, 1, 0, 0};
    L[1] = Layer{{16, 64, 64, 2, 2, 2, 2, 0, 0, 8, 32}, 128, 1, 0, 0};
    L[2] = Layer{{8, 32, 128, 2, 3, 2, 1, 0, 1, 4, 32}, 128, 1, 0, 0};
    L[3] = Layer{{4, 32, 128, 4, 3, 4, 1, 0, 1, 1, 32}, 64, 1, 0, 0};
    L[4] = Layer{{1, 32, 64, 1, 1, 1, 1, 0, 0, 1, 32}, 1, 0, 0, 0};
    uint64_t off = 0;
    for (uint32_t l = 0; l < kLayers; ++l) {
        L[l].w_off = off;
        off += (uint64_t)L[l].cout * L[l].k();
        L[l].b_off = off;
        off += L[l].cout;
    }
}

uint64_t param_count() {
    Layer L[kLayers];
    describe(L);
    return L[kLayers - 1].b_off + L[kLayers - 1].cout;
}

template <class T>
struct DevBuf {
    T* ptr = nullptr;
    uint64_t n = 0;
    int32_t alloc(uint64_t count) {
        release();
        if (int32_t st = cuda_status(cudaMalloc(&ptr, std::max<uint64_t>(count, 1) * sizeof(T)), "cnn allocation"))
            return st;
        n = count;
        return RV_OK;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
    }
};

inline Operand matrix(const void* base, uint32_t rows, uint64_t rs, uint64_t ks) {
    Operand o{};
    o.base = base;
    o.kind = kMatrix;
    o.rows = rows;
    o.rs = rs;
    o.ks = ks;
    return o;
}

inline Operand patch(const void* base, uint32_t kind, uint32_t rows, const Conv& g, uint32_t bf16) {
    Operand o{};
    o.base = base;
    o.kind = kind;
    o.bf16 = bf16;
    o.rows = rows;
    o.g = g;
    return o;
}

inline uint32_t blocks_for(uint64_t n, uint32_t threads, uint32_t cap) {
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, cap));
}

}  // namespace
}  // namespace rv

using namespace rv;

struct rv_cnn {
    rv_context* context = nullptr;
    cudaStream_t stream = nullptr;
    int sms = 152;
    uint32_t max_batch = 0, batch = 0;
    Layer L[kLayers];
    uint64_t params = 0;
    DevBuf<float> p, grad, m, v;
    DevBuf<__nv_bfloat16> pb;              // BF16 copy of p, read by the forward pass
    bool pb_stale = true;
    DevBuf<__nv_bfloat16> act[kLayers - 1];  // post-activation outputs, BF16 NHWC
    DevBuf<float> logits;                  // the head's output
    DevBuf<float> dact[kLayers];           // gradients w.r.t. the layers' outputs
    DevBuf<float> loss;
    DevBuf<uint32_t> status;
    const void* input = nullptr;  // the batch's tiles (BF16), kept for the backward pass
    uint64_t steps = 0;
};

namespace {

int32_t forward_layers(rv_cnn* n, const void* tiles, uint32_t batch) {
    if (n->pb_stale) {
        k_to_bf16<<<blocks_for(n->params, 256, 1024), 256, 0, n->stream>>>(n->p.ptr, n->params, n->pb.ptr);
        if (int32_t st = cuda_status(cudaGetLastError(), "cnn weights")) return st;
        n->pb_stale = false;
    }
    const __nv_bfloat16* x = reinterpret_cast<const __nv_bfloat16*>(tiles);
    for (uint32_t l = 0; l < kLayers; ++l) {
        const Layer& L = n->L[l];
        FwdArgs f{};
        f.x = x;
        f.w = n->pb.ptr + L.w_off;
        f.bias = n->p.ptr + L.b_off;
        f.g = L.g;
        f.m = (uint32_t)(batch * L.pixels());
        f.n = L.cout;
        f.k = L.k();
        f.relu = L.relu;
        f.d = l + 1 < kLayers ? (void*)n->act[l].ptr : (void*)n->logits.ptr;
        f.status = n->status.ptr;
        if (int32_t st = gemm_fwd(n->stream, f)) return st;
        if (l + 1 < kLayers) x = n->act[l].ptr;
    }
    n->input = tiles;
    n->batch = batch;
    return RV_OK;
}

// dact[last] holds dlogits; gradients accumulate into n->grad (zeroed here).
int32_t backward_layers(rv_cnn* n) {
    const uint32_t batch = n->batch;
    if (int32_t st = cuda_status(cudaMemsetAsync(n->grad.ptr, 0, n->params * sizeof(float), n->stream), "cnn grad clear"))
        return st;
    for (uint32_t li = kLayers; li-- > 0;) {
        const Layer& L = n->L[li];
        const uint32_t rows = (uint32_t)(batch * L.pixels());
        float* dz = n->dact[li].ptr;
        if (L.relu) {
            const uint64_t cnt = (uint64_t)rows * L.cout;
            k_relu_grad<<<blocks_for(cnt, 256, 4096), 256, 0, n->stream>>>(dz, n->act[li].ptr, cnt);
            if (int32_t st = cuda_status(cudaGetLastError(), "cnn relu grad")) return st;
        }
        {
            const dim3 grid((L.cout + 31u) / 32u, std::min<uint32_t>(64u, (rows + 255u) / 256u));
            k_bias_grad<<<grid, 1024, 0, n->stream>>>(dz, rows, L.cout, n->grad.ptr + L.b_off);
            if (int32_t st = cuda_status(cudaGetLastError(), "cnn bias grad")) return st;
        }
        const void* x = li == 0 ? n->input : (const void*)n->act[li - 1].ptr;
        const uint32_t bf16 = 1u;
        {  // dW = dZ^T patch(X)
            GemmArgs g{};
            g.a = matrix(dz, L.cout, 1, L.cout);
            g.b = patch(x, kPatchT, L.k(), L.g, bf16);
            g.m = L.cout;
            g.n = L.k();
            g.k = rows;
            g.d = n->grad.ptr + L.w_off;
            g.ldd = L.k();
            g.epilogue = kAtomic;
            g.status = n->status.ptr;
            if (int32_t st = gemm(n->stream, g, n->sms)) return st;
        }
        if (li == 0) break;
        {  // dX = col2im(dZ W)
            float* dx = n->dact[li - 1].ptr;
            const uint64_t xcount = (uint64_t)batch * L.g.h * L.g.w * L.g.c;
            if (int32_t st = cuda_status(cudaMemsetAsync(dx, 0, xcount * sizeof(float), n->stream), "cnn dx clear"))
                return st;
            GemmArgs g{};
            g.a = matrix(dz, rows, L.cout, 1);
            g.b = matrix(n->p.ptr + L.w_off, L.k(), 1, L.k());
            g.m = rows;
            g.n = L.k();
            g.k = L.cout;
            g.d = dx;
            g.epilogue = kCol2im;
            g.out = L.g;
            g.status = n->status.ptr;
            if (int32_t st = gemm(n->stream, g, n->sms)) return st;
        }
    }
    return RV_OK;
}

int32_t check_batch(const rv_cnn* n, uint32_t batch) {
    if (batch == 0 || batch > n->max_batch)
        return set_error_fmt(RV_ERR_INVALID, "rv_cnn: batch of %u tiles (1 .. %u)", batch, n->max_batch);
    return RV_OK;
}

}  // namespace

extern "C" {

uint64_t rv_cnn_param_count(void) { return param_count(); }

int32_t rv_cnn_create(rv_context* context, uint32_t max_batch, uint64_t seed, rv_cnn** out) {
    if (context == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_create: NULL argument");
    *out = nullptr;
    if (max_batch == 0 || max_batch > 65536u)
        return set_error_fmt(RV_ERR_INVALID, "rv_cnn_create: max_batch %u (1 .. 65536)", max_batch);
    rv_cnn* n = new (std::nothrow) rv_cnn;
    if (n == nullptr) return set_error_fmt(RV_ERR_NO_MEMORY, "rv_cnn_create: out of host memory");
    n->context = context;
    n->stream = reinterpret_cast<cudaStream_t>(rv_context_stream(context));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n->sms, cudaDevAttrMultiProcessorCount, dev);
    n->max_batch = max_batch;
    describe(n->L);
    n->params = param_count();
    int32_t st = RV_OK;
    for (DevBuf<float>* b : {&n->p, &n->grad, &n->m, &n->v})
        if (!st) st = b->alloc(n->params);
    if (!st) st = n->pb.alloc(n->params);
    for (uint32_t l = 0; l < kLayers && !st; ++l) {
        const uint64_t count = (uint64_t)max_batch * n->L[l].pixels() * n->L[l].cout;
        st = l + 1 < kLayers ? n->act[l].alloc(count) : n->logits.alloc(count);
        if (!st) st = n->dact[l].alloc(count);
    }
    if (!st) st = n->loss.alloc(1);
    if (!st) st = n->status.alloc(1);
    if (!st) {
        // He-normal weights (std::mt19937_64, Box-Muller), zero biases
        std::vector<float> h(n->params, 0.0F);
        std::mt19937_64 gen(seed);
        const double two_pi = 6.283185307179586;
        for (uint32_t l = 0; l < kLayers; ++l) {
            const double sd = std::sqrt(2.0 / (double)n->L[l].k());
            const uint64_t cnt = (uint64_t)n->L[l].cout * n->L[l].k();
            for (uint64_t i = 0; i < cnt; ++i) {
                const double u1 = ((double)(gen() >> 11) + 1.0) * (1.0 / 9007199254740993.0);
                const double u2 = (double)(gen() >> 11) * (1.0 / 9007199254740992.0);
                h[n->L[l].w_off + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2));
            }
        }
        st = cuda_status(cudaMemcpyAsync(n->p.ptr, h.data(), n->params * sizeof(float), cudaMemcpyHostToDevice, n->stream),
                         "cnn parameters");
        if (!st) st = cuda_status(cudaMemsetAsync(n->m.ptr, 0, n->params * sizeof(float), n->stream), "cnn adam");
        if (!st) st = cuda_status(cudaMemsetAsync(n->v.ptr, 0, n->params * sizeof(float), n->stream), "cnn adam");
        if (!st) st = cuda_status(cudaMemsetAsync(n->status.ptr, 0, sizeof(uint32_t), n->stream), "cnn status");
        if (!st) st = cuda_status(cudaStreamSynchronize(n->stream), "cnn setup");
    }
    if (st) {
        rv_cnn_destroy(n);
        return st;
    }
    *out = n;
    return clear_error();
}

int32_t rv_cnn_destroy(rv_cnn* n) {
    if (n == nullptr) return RV_OK;
    if (n->stream) cudaStreamSynchronize(n->stream);
    for (DevBuf<float>* b : {&n->p, &n->grad, &n->m, &n->v, &n->loss, &n->logits}) b->release();
    n->pb.release();
    for (uint32_t l = 0; l < kLayers; ++l) {
        if (l + 1 < kLayers) n->act[l].release();
        n->dact[l].release();
    }
    n->status.release();
    delete n;
    return clear_error();
}

int32_t rv_cnn_set_params(rv_cnn* n, const float* host, uint64_t count) {
    if (n == nullptr || host == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_set_params: NULL argument");
    if (count != n->params)
        return set_error_fmt(RV_ERR_INVALID, "rv_cnn_set_params: %llu values for %llu parameters",
                             (unsigned long long)count, (unsigned long long)n->params);
    if (int32_t st = cuda_status(cudaMemcpyAsync(n->p.ptr, host, count * sizeof(float), cudaMemcpyHostToDevice, n->stream),
                                 "cnn set params"))
        return st;
    n->pb_stale = true;
    return cuda_status(cudaStreamSynchronize(n->stream), "cnn set params") ? RV_ERR_CUDA : clear_error();
}

static int32_t read_vec(rv_cnn* n, const float* dev, float* host, uint64_t count, const char* what) {
    if (n == nullptr || host == nullptr) return set_error_fmt(RV_ERR_INVALID, "%s: NULL argument", what);
    if (count != n->params)
        return set_error_fmt(RV_ERR_INVALID, "%s: %llu values for %llu parameters", what, (unsigned long long)count,
                             (unsigned long long)n->params);
    if (int32_t st = cuda_status(cudaMemcpyAsync(host, dev, count * sizeof(float), cudaMemcpyDeviceToHost, n->stream), what))
        return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(n->stream), what)) return st;
    return clear_error();
}

int32_t rv_cnn_get_params(rv_cnn* n, float* host, uint64_t count) {
    return read_vec(n, n ? n->p.ptr : nullptr, host, count, "rv_cnn_get_params");
}

int32_t rv_cnn_get_grads(rv_cnn* n, float* host, uint64_t count) {
    return read_vec(n, n ? n->grad.ptr : nullptr, host, count, "rv_cnn_get_grads");
}

void* rv_cnn_stream(const rv_cnn* n) { return n ? (void*)n->stream : nullptr; }

int32_t rv_cnn_set_stream(rv_cnn* n, void* stream) {
    if (n == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_set_stream: NULL");
    if (int32_t st = cuda_status(cudaStreamSynchronize(n->stream), "cnn stream")) return st;
    n->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : reinterpret_cast<cudaStream_t>(rv_context_stream(n->context));
    return clear_error();
}

int32_t rv_cnn_forward(rv_cnn* n, const void* tiles_dev, uint32_t batch, float* logits_dev, uint64_t logits_len) {
    if (n == nullptr || tiles_dev == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_forward: NULL argument");
    if (int32_t st = check_batch(n, batch)) return st;
    const uint64_t out = (uint64_t)batch * RV_CNN_CELLS;
    if (logits_dev != nullptr && logits_len < out)
        return set_error_fmt(RV_ERR_INVALID, "rv_cnn_forward: logits buffer of %llu for %llu",
                             (unsigned long long)logits_len, (unsigned long long)out);
    if (int32_t st = forward_layers(n, tiles_dev, batch)) return st;
    if (logits_dev != nullptr)
        if (int32_t st = cuda_status(cudaMemcpyAsync(logits_dev, n->logits.ptr, out * sizeof(float),
                                                     cudaMemcpyDeviceToDevice, n->stream),
                                     "cnn logits"))
            return st;
    return clear_error();
}

int32_t rv_cnn_backward(rv_cnn* n, const float* dlogits_dev, uint64_t dlogits_len) {
    if (n == nullptr || dlogits_dev == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_backward: NULL argument");
    if (n->batch == 0) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_backward: no forward pass to differentiate");
    const uint64_t out = (uint64_t)n->batch * RV_CNN_CELLS;
    if (dlogits_len < out) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_backward: %llu gradients for %llu logits",
                                                (unsigned long long)dlogits_len, (unsigned long long)out);
    if (int32_t st = cuda_status(cudaMemcpyAsync(n->dact[kLayers - 1].ptr, dlogits_dev, out * sizeof(float),
                                                 cudaMemcpyDeviceToDevice, n->stream),
                                 "cnn dlogits"))
        return st;
    if (int32_t st = backward_layers(n)) return st;
    return clear_error();
}

int32_t rv_cnn_train_step(rv_cnn* n, const void* tiles_dev, const float* labels_dev, uint32_t batch,
                          const rv_cnn_train_config* cfg, float* loss_host) {
    if (n == nullptr || tiles_dev == nullptr || labels_dev == nullptr || cfg == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_cnn_train_step: NULL argument");
    if (int32_t st = check_batch(n, batch)) return st;
    if (!(cfg->learning_rate > 0.0F) || !(cfg->beta1 >= 0.0F && cfg->beta1 < 1.0F) ||
        !(cfg->beta2 >= 0.0F && cfg->beta2 < 1.0F) || !(cfg->epsilon > 0.0F) || !(cfg->pos_weight > 0.0F))
        return set_error_fmt(RV_ERR_INVALID, "rv_cnn_train_step: learning rate, betas, epsilon or pos_weight out of range");
    if (int32_t st = forward_layers(n, tiles_dev, batch)) return st;
    const uint32_t out = batch * RV_CNN_CELLS;
    if (int32_t st = cuda_status(cudaMemsetAsync(n->loss.ptr, 0, sizeof(float), n->stream), "cnn loss")) return st;
    k_bce<<<blocks_for(out, 256, 1024), 256, 0, n->stream>>>(n->logits.ptr, labels_dev, out, cfg->pos_weight,
                                                           n->dact[kLayers - 1].ptr, n->loss.ptr);
    if (int32_t st = cuda_status(cudaGetLastError(), "cnn loss")) return st;
    if (int32_t st = backward_layers(n)) return st;
    n->steps += 1;
    AdamArgs a{cfg->learning_rate, cfg->beta1, cfg->beta2, cfg->epsilon,
               (float)(1.0 - std::pow((double)cfg->beta1, (double)n->steps)),
               (float)(1.0 - std::pow((double)cfg->beta2, (double)n->steps)), cfg->weight_decay};
    k_adam<<<blocks_for(n->params, 256, 1024), 256, 0, n->stream>>>(n->p.ptr, n->grad.ptr, n->m.ptr, n->v.ptr, n->params, a,
                                                                   n->pb.ptr);
    if (int32_t st = cuda_status(cudaGetLastError(), "cnn adam")) return st;
    if (loss_host != nullptr) {
        if (int32_t st = cuda_status(cudaMemcpyAsync(loss_host, n->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, n->stream),
                                     "cnn loss read"))
            return st;
        if (int32_t st = cuda_status(cudaStreamSynchronize(n->stream), "cnn train step")) return st;
    }
    return clear_error();
}

int32_t rv_cnn_status(rv_cnn* n, uint32_t* timeouts) {
    if (n == nullptr || timeouts == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_cnn_status: NULL argument");
    if (int32_t st = cuda_status(cudaMemcpyAsync(timeouts, n->status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, n->stream),
                                 "cnn status"))
        return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(n->stream), "cnn status")) return st;
    if (*timeouts) return set_error_fmt(RV_ERR_TIMEOUT, "rv_cnn: %u CTAs gave up waiting on the tensor cores", *timeouts);
    return clear_error();
}

// A plain GEMM through the same kernel, for testing it on its own:
// D[m][n] = sum_k A[m][k] B[n][k] (FP32 row-major in and out, rounded to
// BF16 on the way into the tensor cores).
int32_t rv_gemm_bf16(void* stream, const float* a_dev, const float* b_dev, uint32_t m, uint32_t n, uint32_t k,
                     float* d_dev, uint32_t* status_dev) {
    if (a_dev == nullptr || b_dev == nullptr || d_dev == nullptr || status_dev == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_gemm_bf16: NULL argument");
    if (m == 0 || n == 0 || k == 0) return clear_error();
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    GemmArgs g{};
    g.a = matrix(a_dev, m, k, 1);
    g.b = matrix(b_dev, n, k, 1);
    g.m = m;
    g.n = n;
    g.k = k;
    g.d = d_dev;
    g.ldd = n;
    g.epilogue = kStore;
    g.status = status_dev;
    if (int32_t st = gemm(reinterpret_cast<cudaStream_t>(stream), g, sms)) return st;
    return clear_error();
}

}  // extern "C"
