// Fine stage on the tensor cores (the chain's fast mode): the resampler's
// dot products as split-precision BF16 GEMMs on tcgen05, FP32 accumulation in
// tensor memory, then the NCO rotation.
//
// With the 2D tiling of fine_tiles.cu (output j = row * P' + column a, row
// b's input window row 0's shifted by b Dp samples), a group of W = 32
// columns a0 .. a0 + 31 over 128 rows is one GEMM:
//   out[b][c] = sum_m x[s_b + m] * B_c[m],   s_b = b Dp + n(a0) - (T - 1),
//   B_c[m] = g_{a0 + c}[off_c + T - 1 - m]  (zero outside the T taps),
// where g_a is column a's blended tap vector and off_c = n(a0 + c) - n(a0): a
// banded complex matrix, fixed per receiver and group. In real form with the
// K index interleaving (re, im) of each input sample, A's rows are the
// channel stream itself and B has one row per output part:
//   re row: ( Re g, -Im g ),  im row: ( Im g, Re g )  per input sample.
// Operands are split x = hi + lo (both BF16, lo = bf16(x - hi)), and the
// tensor cores accumulate hi*hi + lo*hi + hi*lo (lo*lo, below 2^-16
// relative, is dropped): each product carries about 17 significant bits,
// close to the FP32 sum it replaces. Outputs are checked against the
// bit-exact chain to a stated relative-RMS tolerance, never bit for bit.
//
// B is built once per receiver (k_fine_tc_tables) as the shared-memory image
// of each 64-element K chunk in the 128-byte swizzled K-major layout, hi rows
// then lo rows, so a chunk's B is one bulk copy and one 2 kN-row operand. The
// CTA is warp-specialised, one per SM, persistent over a static share of the
// tiles (sorted by cost on the host):
//   * eight converter warps load a chunk's samples straight from the channel
//     ring into registers one chunk ahead, split them into hi / lo and store
//     the swizzled A images into a ring of four stages; their thread 0 also
//     bulk-copies the chunk's B onto the stage's full barrier;
//   * one MMA warp waits for a full stage and issues, per 16-wide K step,
//     hi * (B hi | B lo) at N = 2 kN and lo * B hi at N = kN into one
//     accumulator (columns 0 .. kN - 1 get hi*hi + lo*hi, kN .. 2 kN - 1
//     hi*lo), committing the stage's empty barrier; after a tile's last chunk
//     it commits the accumulator, double-buffered in tensor memory;
//   * four epilogue warps (one per TMEM lane quarter) read a finished
//     accumulator, free it, add its halves, rotate by the NCO (table reads
//     batched ahead of the stores) and write the fine ring.
// Every mbarrier wait is bounded; a wait that runs out stops every role,
// counts in the status word, the converters wait (bounded) for their B
// copies, and the MMA warp waits (bounded) for its committed MMAs before the
// tensor memory is freed.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "receivers.cuh"
#include "tc.cuh"

namespace rv {
namespace {

constexpr uint32_t kW = kFineTcColumns;        // outputs (columns) per GEMM tile
constexpr uint32_t kN = 2u * kW;               // GEMM N: (re, im) per output
constexpr uint32_t kRowsTc = kFineTcRows;      // GEMM M
constexpr uint32_t kKc = 64;                   // real K per chunk: 32 complex samples
constexpr uint32_t kA = kRowsTc * kKc * 2u;    // one A part (hi or lo), bytes
constexpr uint32_t kB = kN * kKc * 2u;         // one B part
constexpr uint32_t kTmemCols = 2u * kN;  // one accumulator: the two halves below
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t idesc = tc::instr_desc_f16(1u, kRowsTc, kN);
constexpr uint32_t idesc_wide = tc::instr_desc_f16(1u, kRowsTc, 2u * kN);

__device__ __forceinline__ uint32_t bf16_bits(float x) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
}

// B tables: for group g and chunk k, kN rows x kKc in the K-major core-matrix
// image, the hi part then the lo part (2 kB bytes).
__global__ void k_fine_tc_tables(const float2* __restrict__ lerped, uint32_t T, uint32_t period, uint32_t P,
                                 uint32_t step_whole, uint32_t step_rem, uint32_t fd, uint32_t groups,
                                 uint32_t chunks, uint16_t* __restrict__ out) {
    const uint64_t per_chunk = (uint64_t)kN * kKc;  // elements of one part
    const uint64_t total = (uint64_t)groups * chunks * per_chunk;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)((e / kKc) % kN), kk = (uint32_t)(e % kKc);
        const uint64_t gk = e / per_chunk;
        const uint32_t k = (uint32_t)(gk % chunks), g = (uint32_t)(gk / chunks);
        const uint32_t c = r >> 1, im_row = r & 1u;
        const uint32_t a0 = g * kW, a = a0 + c;
        float v = 0.0F;
        if (a < P) {
            const uint32_t n_a0 = a0 * step_whole + (uint32_t)((uint64_t)a0 * step_rem / fd);
            const uint32_t n_a = a * step_whole + (uint32_t)((uint64_t)a * step_rem / fd);
            const int64_t m = (int64_t)((k * kKc + kk) >> 1);
            const int64_t q = (int64_t)(n_a - n_a0) + (int64_t)T - 1 - m;
            if (q >= 0 && q < (int64_t)T) {
                const float2 tap = lerped[(uint64_t)q * period + (a % period)];
                const bool x_im = (kk & 1u) != 0;
                v = im_row ? (x_im ? tap.x : tap.y) : (x_im ? -tap.y : tap.x);
            }
        }
        const float hi = __bfloat162float(__float2bfloat16_rn(v));
        const uint64_t base = gk * 2u * per_chunk;
        const uint32_t off = tc::sw128_offset(r, kk) >> 1;  // in elements
        out[base + off] = (uint16_t)bf16_bits(v);
        out[base + per_chunk + off] = (uint16_t)bf16_bits(v - hi);
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// Warp roles: eight converter warps, one MMA warp, four epilogue warps (one
// per TMEM lane quarter: warp w reads lanes 32 (w % 4) ..).
constexpr uint32_t kConvWarps = 8;
constexpr uint32_t kConvThreads = kConvWarps * 32u;
constexpr uint32_t kMmaWarp = kConvWarps;
constexpr uint32_t kWarpsTc = kMmaWarp + 1u + 4u;
constexpr uint32_t kRing = 4;  // stages
constexpr uint32_t kItems = kRowsTc / 8u;  // items a converter thread takes per chunk

// A chunk's stage: the hi and lo BF16 images of A (kA bytes each), then B as
// it lies in the tables (hi rows then lo rows: one 2 kN-row operand).
constexpr uint32_t kBOffset = 2u * kA;
constexpr uint32_t kStage = kBOffset + 2u * kB;
static_assert(kKc == 64u && kA % 1024u == 0u && kB % 1024u == 0u && kStage % 1024u == 0u,
              "swizzled operands: 128-byte rows, every image on a 1024-byte boundary");
static_assert(kConvWarps * 4u == kKc / 2u, "converter warp w takes samples 4 w .. 4 w + 3 of a chunk");

// The tile a walk is in, fixed over its chunks. Ring offsets are taken
// modulo 2^32 and then masked: the ring length divides 2^32.
struct TileWalk {
    const RxDev* rxs;
    const FineTile* tiles;
    const float2* chan;  // every channel's ring
    uint32_t ntiles, u, k, chunks, rows;
    const float2* ring;  // the receiver's channel ring
    uint32_t mask;       // ring samples - 1
    uint32_t first;      // ring offset (before masking) of row 0's first sample in chunk 0
    uint32_t step;       // samples between rows
    const uint8_t* btab; // the group's B chunks
    __device__ bool start(const RxDev* r, const FineTile* t, uint32_t n, const float2* c) {
        rxs = r, tiles = t, ntiles = n, chan = c, u = blockIdx.x;
        return enter();
    }
    __device__ bool enter() {  // chunk 0 of tile u, skipping empty tiles
        for (; u < ntiles; u += gridDim.x) {
            const FineTile t = tiles[u];
            const RxDev& rx = rxs[t.rx];
            chunks = rx.tc_chunks;
            if (chunks == 0) continue;
            const uint32_t n_a0 = t.a0 * rx.step_whole + (uint32_t)((uint64_t)t.a0 * rx.step_rem / rx.out_rate);
            step = (uint32_t)rx.row_step;
            first = n_a0 - (rx.taps - 1u) + (uint32_t)t.row0 * step;
            ring = chan + rx.chan_base;
            mask = rx.chan_mask;
            rows = t.rows;
            btab = reinterpret_cast<const uint8_t*>(rx.tc_b) + (uint64_t)(t.a0 / kW) * chunks * 2u * kB;
            k = 0;
            return true;
        }
        return false;
    }
    __device__ bool next() {
        if (++k < chunks) return true;
        u += gridDim.x;
        return enter();
    }
};

// A converter thread's samples of one chunk: in item i (row octet i) lane l
// of warp w owns row 8 i + l / 4, sample 4 w + l % 4 (a warp's load reads
// four consecutive samples of eight rows: eight whole sectors). Rows past the
// tile read row 0's sample (their MMA rows are never read).
__device__ __forceinline__ void load_chunk(float2 (&x)[kItems], const TileWalk& w, uint32_t warp, uint32_t lane) {
    const uint32_t r0 = lane >> 2;
    const uint32_t b = w.first + r0 * w.step + w.k * (kKc / 2u) + 4u * warp + (lane & 3u);
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t at = (8u * i + r0 < w.rows) ? b + i * 8u * w.step : b - r0 * w.step;
        x[i] = __ldg(w.ring + (at & w.mask));
    }
}

// B is streamed once per tile: its lines go first when L2 needs room, so the
// channel rings the tiles re-read stay resident.
__device__ __forceinline__ void bulk_copy_stream(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    uint64_t policy;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(policy));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;\n" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(mbar), "l"(policy)
        : "memory");
}
__device__ __forceinline__ void arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}

// Barrier 1 over the converter threads only, returning whether any of them
// passed `v` (so every converter takes the same branch after it).
__device__ __forceinline__ bool converters_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(kConvThreads)
        : "memory");
    return r != 0u;
}

// Two floats as a BF16 pair, rounded to nearest even with integer arithmetic
// (finite inputs: the lo parts of finite samples).
__device__ __forceinline__ uint32_t pack2_int(float a, float b) {
    const uint32_t ua = __float_as_uint(a), ub = __float_as_uint(b);
    const uint32_t ra = ua + 0x7FFFu + ((ua >> 16) & 1u), rb = ub + 0x7FFFu + ((ub >> 16) & 1u);
    return __byte_perm(ra, rb, 0x7632);
}

// The thread's samples, split hi / lo, into the images of stage `st`: its
// four-byte stores of the (re, im) pair fill, across the warp, 128 bytes
// (eight rows' pieces of one swizzled K group: no bank conflict). hi is the
// rounded pair (one conversion), lo the remainder rounded by integer
// arithmetic.
__device__ __forceinline__ void store_chunk(uint8_t* st, const float2 (&x)[kItems], uint32_t warp, uint32_t lane) {
    const uint32_t kcol = 8u * warp + 2u * (lane & 3u);
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t row = 8u * i + (lane >> 2);
        const __nv_bfloat162 h = __floats2bfloat162_rn(x[i].x, x[i].y);
        const uint32_t hb = *reinterpret_cast<const uint32_t*>(&h);
        const float h0 = __uint_as_float(hb << 16), h1 = __uint_as_float(hb & 0xFFFF0000u);
        const uint32_t off = tc::sw128_offset(row, kcol);
        *reinterpret_cast<uint32_t*>(st + off) = hb;
        *reinterpret_cast<uint32_t*>(st + kA + off) = pack2_int(x[i].x - h0, x[i].y - h1);
    }
}

// Bounded wait shared by every role: false once the limit ran out or
// another role gave up (then this one stops too).
__device__ __forceinline__ bool wait_or_abort(uint32_t mbar, uint32_t parity, volatile uint32_t* abort_flag) {
    for (uint32_t round = 0; round < 64u; ++round) {
        if (tc::wait_parity(mbar, parity, kWaitLimit / 64u)) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1u;
    return false;
}

// Accumulator layout (kTmemCols columns a buffer): columns 0 .. kN - 1 hold
// hi*hi + lo*hi, columns kN .. 2 kN - 1 hi*lo (the same MMA as hi*hi, with
// B's lo rows as the second half of N).
__global__ void __launch_bounds__(kWarpsTc * 32u, 1)
k_fine_tc(const RxDev* __restrict__ rxs, const FineTile* __restrict__ tiles, uint32_t ntiles,
          const float2* __restrict__ chan, uint32_t* queue, const uint32_t* dyn, uint32_t* status) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* const full = reinterpret_cast<uint64_t*>(sm + kRing * kStage);
    uint64_t* const empty = full + kRing;
    uint64_t* const acc_full = empty + kRing;
    uint64_t* const acc_empty = acc_full + 2;
    __shared__ uint32_t s_tmem;
    __shared__ volatile uint32_t s_abort;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    (void)queue;
    if (dyn != nullptr) ntiles = *dyn;
    if (warp == kMmaWarp) tc::tmem_alloc(tc::smem_addr(&s_tmem), 2u * kTmemCols);
    if (tid == 0) {
        for (uint32_t b = 0; b < kRing; ++b) {
            tc::mbar_init(tc::smem_addr(full + b), kConvWarps + 1u);  // converter warps + B's expect
            tc::mbar_init(tc::smem_addr(empty + b), 1);
        }
        for (uint32_t b = 0; b < 2u; ++b) {
            tc::mbar_init(tc::smem_addr(acc_full + b), 1);
            tc::mbar_init(tc::smem_addr(acc_empty + b), 128);
        }
        tc::mbar_fence_init();
        // the swizzled images need 1024-byte aligned stages: otherwise stop
        s_abort = (tc::smem_addr(sm) & 1023u) != 0u ? 1u : 0u;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = s_tmem;
    // every role walks the same tiles: blockIdx.x, + gridDim.x, ...
    if (warp < kConvWarps) {
        // converters: chunk `it` is stored into stage it % kRing (once its
        // previous chunk has left the MMAs) while chunk it + 1 loads; thread
        // 0 also copies the chunk's B
        TileWalk w;
        bool more = w.start(rxs, tiles, ntiles, chan);
        float2 cur[kItems], nxt[kItems];
        if (more) load_chunk(nxt, w, warp, lane);
        uint32_t it = 0;
        for (; more; ++it) {
            const uint32_t slot = it % kRing;
            bool ok = true;
            if (it >= kRing) ok = wait_or_abort(tc::smem_addr(empty + slot), ((it / kRing) - 1u) & 1u, &s_abort);
            if (converters_any(!ok || s_abort)) break;
            uint8_t* const st = sm + slot * kStage;
            if (tid == 0) {
                arrive_expect_tx(tc::smem_addr(full + slot), 2u * kB);
                bulk_copy_stream(tc::smem_addr(st + kBOffset), w.btab + (uint64_t)w.k * 2u * kB, 2u * kB, tc::smem_addr(full + slot));
            }
#pragma unroll
            for (uint32_t i = 0; i < kItems; ++i) cur[i] = nxt[i];
            more = w.next();
            if (more) load_chunk(nxt, w, warp, lane);
            store_chunk(st, cur, warp, lane);
            tc::fence_async_smem();
            __syncwarp();  // the warp's stores before its one arrival
            if (lane == 0) mbar_arrive(tc::smem_addr(full + slot));
        }
        // after a stop, B copies still landing finish before the stages go
        if (tid == 0)
            for (uint32_t j = it > kRing ? it - kRing : 0u; j < it; ++j)
                tc::wait_parity(tc::smem_addr(full + j % kRing), (j / kRing) & 1u, kWaitLimit);
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            uint32_t it = 0, tcount = 0;
            for (uint32_t u = blockIdx.x; u < ntiles && !s_abort; u += gridDim.x, ++tcount) {
                const FineTile t = tiles[u];
                const uint32_t chunks = rxs[t.rx].tc_chunks;
                const uint32_t acc = tcount & 1u, d = tmem + acc * kTmemCols;
                if (tcount >= 2u && !wait_or_abort(tc::smem_addr(acc_empty + acc), ((tcount >> 1) - 1u) & 1u, &s_abort))
                    break;
                tc::fence_after();
                bool ok = true;
                for (uint32_t c = 0; c < chunks; ++c, ++it) {
                    const uint32_t slot = it % kRing;
                    if (!wait_or_abort(tc::smem_addr(full + slot), (it / kRing) & 1u, &s_abort)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after();
                    const uint32_t a_hi = tc::smem_addr(sm + slot * kStage), a_lo = a_hi + kA;
                    const uint32_t b = a_hi + kBOffset;
#pragma unroll
                    for (uint32_t s = 0; s < kKc / 16u; ++s) {
                        const uint32_t o = 32u * s;
                        // hi * (B hi | B lo) into columns 0 .. 2 kN - 1, then lo * B hi into 0 .. kN - 1
                        tc::mma_f16(d, tc::smem_desc_sw128(a_hi + o), tc::smem_desc_sw128(b + o), idesc_wide,
                                    (c > 0u || s > 0u) ? 1u : 0u);
                        tc::mma_f16(d, tc::smem_desc_sw128(a_lo + o), tc::smem_desc_sw128(b + o), idesc, 1u);
                    }
                    tc::commit(tc::smem_addr(empty + slot));  // the stage is free once these MMAs finish
                }
                if (!ok) break;
                tc::commit(tc::smem_addr(acc_full + acc));  // the tile's accumulator is complete
            }
            // the MMAs this warp committed finish before the tensor memory goes
            if (it > 0) wait_or_abort(tc::smem_addr(empty + (it - 1u) % kRing), ((it - 1u) / kRing) & 1u, &s_abort);
        }
        __syncwarp();
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31
        const uint32_t quarter = warp & 3u, row = quarter * 32u + lane;
        uint32_t tcount = 0;
        for (uint32_t u = blockIdx.x; u < ntiles && !s_abort; u += gridDim.x, ++tcount) {
            const FineTile t = tiles[u];
            const RxDev& rx = rxs[t.rx];
            const uint32_t acc = tcount & 1u;
            if (!wait_or_abort(tc::smem_addr(acc_full + acc), (tcount >> 1) & 1u, &s_abort)) break;
            tc::fence_after();
            float v[kN];
            const uint32_t base = tmem + ((quarter * 32u) << 16) + acc * kTmemCols;
#pragma unroll
            for (uint32_t col = 0; col < kN; col += 16u) {
                float lo[16];
                tc::tmem_ld16(base + col, v + col);
                tc::tmem_ld16(base + kN + col, lo);
#pragma unroll
                for (uint32_t i = 0; i < 16u; ++i) v[col + i] += lo[i];
            }
            tc::fence_before();
            mbar_arrive(tc::smem_addr(acc_empty + acc));  // the accumulator may be overwritten
            if (row < t.rows) {
                const uint64_t jrow = (t.row0 + row) * rx.tile_period + t.a0;
                const float2* nco = rx.nco;
                const uint64_t delta = rx.nco_delta;
                const uint32_t log2 = rx.nco_log2, mask = rx.fine_mask;
                float2* fine = rx.fine;
                // sixteen table reads in flight before the first store (the
                // stores could alias them, so they are not reordered past it)
#pragma unroll
                for (uint32_t h = 0; h < kW; h += 16u) {
                    float2 rot[16];
#pragma unroll
                    for (uint32_t c = 0; c < 16u; ++c) {
                        const uint64_t phi = delta * (jrow + h + c);
                        rot[c] = __ldg(nco + ((log2 == 0) ? 0u : ((uint32_t)(phi >> 32) >> (32u - log2))));
                    }
#pragma unroll
                    for (uint32_t c = 0; c < 16u; ++c) {
                        const uint32_t col = h + c;
                        const uint64_t j = jrow + col;
                        if (col >= t.width || j < t.first || j >= t.end) continue;
                        const float re = v[2 * col], im = v[2 * col + 1];
                        fine[(uint32_t)j & mask] = make_float2(re * rot[c].x - im * rot[c].y, re * rot[c].y + im * rot[c].x);
                    }
                }
            }
        }
    }
    if (tid == 0 && s_abort) atomicAdd(status, 1u);
    tc::fence_before();
    __syncthreads();
    if (warp == kMmaWarp) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, 2u * kTmemCols);
    }
}

constexpr uint32_t kSmemWs = kRing * kStage + 128u;  // + full, empty, acc_full, acc_empty barriers

}  // namespace

uint32_t fine_tc_chunks(uint32_t taps, uint32_t P, uint32_t step_whole, uint32_t step_rem, uint32_t fd) {
    // the widest group's band: off of its last column plus T samples
    uint32_t widest = 0;
    for (uint32_t a0 = 0; a0 < P; a0 += kW) {
        const uint32_t last = (a0 + kW - 1u < P) ? a0 + kW - 1u : P - 1u;
        const uint32_t n0 = a0 * step_whole + (uint32_t)((uint64_t)a0 * step_rem / fd);
        const uint32_t n1 = last * step_whole + (uint32_t)((uint64_t)last * step_rem / fd);
        if (n1 - n0 > widest) widest = n1 - n0;
    }
    const uint32_t samples = widest + taps;
    return (samples + kKc / 2u - 1u) / (kKc / 2u);
}

uint64_t fine_tc_table_elements(uint32_t P, uint32_t chunks) {
    return (uint64_t)((P + kW - 1u) / kW) * chunks * 2u * kN * kKc;
}

int32_t launch_fine_tc_tables(cudaStream_t s, const float2* lerped, uint32_t T, uint32_t period, uint32_t P,
                              uint32_t step_whole, uint32_t step_rem, uint32_t fd, uint32_t chunks, uint16_t* out) {
    const uint32_t groups = (P + kW - 1u) / kW;
    const uint64_t n = (uint64_t)groups * chunks * kN * kKc;
    const uint32_t blocks = (uint32_t)((n + 255u) / 256u < 65535u ? (n + 255u) / 256u : 65535u);
    k_fine_tc_tables<<<blocks, 256, 0, s>>>(lerped, T, period, P, step_whole, step_rem, fd, groups, chunks, out);
    return cuda_status(cudaGetLastError(), "fine tc tables");
}

int32_t launch_fine_tc(cudaStream_t s, const RxDev* rxs, const FineTile* tiles, uint32_t ntiles, const float2* chan,
                       uint32_t* queue, const uint32_t* dyn, uint32_t* status) {
    if (ntiles == 0) return RV_OK;
    if (int32_t st = ensure_shared((const void*)k_fine_tc, kSmemWs, "fine tc shared memory")) return st;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t cap = (uint32_t)sms;  // one CTA an SM
    const uint32_t grid = dyn != nullptr ? cap : (ntiles < cap ? ntiles : cap);
    k_fine_tc<<<grid, kWarpsTc * 32u, kSmemWs, s>>>(rxs, tiles, ntiles, chan, queue, dyn, status);
    return cuda_status(cudaGetLastError(), "fine tc");
}

}  // namespace rv
