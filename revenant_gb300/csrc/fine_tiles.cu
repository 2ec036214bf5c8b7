// Fine stage as 2D tiles: pattern phase x period rows.
//
// reference_vrx_fine (core/dsp/vrx_reference.cpp:489-620) computes fine
// output j of a receiver as  sum_q x[n(j) - q] * tap_{phase(j)}[q]  (ascending
// q, complex, taps blended per output), then rotates it by the NCO. With
// Fc the channel rate and Fd the demodulator rate, n(j) = floor(j Fc / Fd) and
// the (phase, blend) pair depends only on (j Fc) mod Fd, which repeats every
// P = Fd / gcd(Fc, Fd) outputs, and so does it every P' = k P. Writing
// j = b P' + a (row b, column a; k makes rows at least 48 outputs long):
//   * the blended tap column of output j is a mod P, so every row of a column
//     uses the same T taps;
//   * n(b P' + a) = b Dp + n(a) with Dp = P' Fc / Fd, so row b's input window
//     is row 0's shifted by b Dp samples.
// A tile is a block of columns [a0, a0 + width) over a range of rows. Its
// slice of the blended table ([T][width]) stays in shared memory for the whole
// tile; the rows pass through in chunks, each row's input segment (the samples
// its columns need, n(a0 + width - 1) - n(a0) + T of them) copied into shared
// memory with cp.async, the next chunk while the current one is computed.
// Chunks are 16 rows; a thread owns one row and R adjacent columns, so a
// half-warp reads one tap (broadcast) and 16 rows' samples (an odd row stride
// keeps them in distinct banks) per column and tap. The per-output sum runs
// over q in ascending order with a rounded multiply and a rounded add per
// step, so every output keeps the reference's bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "receivers.cuh"

namespace rv {
namespace {

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void add_pair(uint64_t& acc, float lo, float hi) {
    asm("{\n .reg .b64 t;\n mov.b64 t, {%1, %2};\n add.rn.ftz.f32x2 %0, %0, t;\n}\n" : "+l"(acc) : "f"(lo), "f"(hi));
}
__device__ __forceinline__ void unpack_pair(uint64_t acc, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc));
}

__device__ __forceinline__ uint32_t next_tile(uint32_t* queue, uint32_t* slot) {
    __syncthreads();
    if (threadIdx.x == 0) *slot = atomicAdd(queue, 1u);
    __syncthreads();
    return *slot;
}

// Rows [r0, r0 + nrows) of the tile into `buf`, row k at buf + k * stride:
// the channel samples from (row0 + r0 + k) Dp + n(a0) - (T - 1) on.
__device__ __forceinline__ void stage_rows(float2* buf, const RxDev& rx, const float2* __restrict__ chan,
                                           uint64_t first_row, uint32_t nrows, uint32_t n_a0) {
    const uint32_t L = rx.tile_seg, Lp = rx.tile_stride;
    for (uint32_t k = 0; k < nrows; ++k) {
        const uint64_t s0 = (first_row + k) * rx.row_step + n_a0 - (rx.taps - 1u);
        float2* dst = buf + k * Lp;
        for (uint32_t i = threadIdx.x; i < L; i += blockDim.x)
            cp_async8(dst + i, chan + rx.chan_base + (uint32_t)((s0 + i) & rx.chan_mask));
    }
}

// Thread (row, slot): one row of the chunk and columns slot*R .. slot*R+R-1.
// A half-warp holds 16 rows of the same columns: its tap loads are one
// broadcast, its sample loads stride the odd row stride (no bank conflicts).
// The table slice holds taps in pairs: float2 (((q >> 1) * Ap + c) * 2 +
// (q & 1)), so one 16-byte load brings taps q and q + 1 of a column.
template <int R>
__device__ __forceinline__ void compute_cols(const float2* tab, const float2* buf, const RxDev& rx,
                                             const FineTile& t, uint64_t first_row, uint32_t nrows, uint32_t row,
                                             uint32_t c0, uint32_t n_a0) {
    const uint32_t T = rx.taps, Ap = rx.tile_cols, Lp = rx.tile_stride;
    const float2* sp[R];
    uint64_t j[R];
    bool act[R];
    const uint64_t jrow = (first_row + row) * rx.tile_period + t.a0;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const uint32_t c = c0 + (uint32_t)k;
        const uint32_t a = t.a0 + (c < t.width ? c : t.width - 1u);  // past the block: any column, result unused
        const uint32_t off = a * rx.step_whole + (uint32_t)((uint64_t)a * rx.step_rem / rx.out_rate) - n_a0;
        sp[k] = buf + row * Lp + off + T - 1u;  // sp[k][-q] = x[n(j) - q]
        j[k] = jrow + c;
        act[k] = row < nrows && c < t.width && j[k] >= t.first && j[k] < t.end;
    }
    // (re, im) of each output's sum as one packed pair: the product's two
    // parts are rounded scalar operations, the two accumulating adds one
    // add.rn.ftz.f32x2 (lane for lane the scalar add)
    uint64_t acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = 0;
    // blocks of four taps, every operand loaded before the first multiply;
    // the sums still take q in ascending order
    const float4* tq = reinterpret_cast<const float4*>(tab) + c0;
    uint32_t q = 0;
#pragma unroll 1
    for (; q + 4u <= T; q += 4u) {
        float4 t01[R], t23[R];
        float2 sv[4][R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            t01[k] = tq[k];
            t23[k] = tq[Ap + k];
#pragma unroll
            for (int u = 0; u < 4; ++u) sv[u][k] = sp[k][-u];
        }
        tq += 2u * Ap;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            sp[k] -= 4;
            const float2 tv[4] = {make_float2(t01[k].x, t01[k].y), make_float2(t01[k].z, t01[k].w),
                                  make_float2(t23[k].x, t23[k].y), make_float2(t23[k].z, t23[k].w)};
#pragma unroll
            for (int u = 0; u < 4; ++u)
                add_pair(acc[k], sv[u][k].x * tv[u].x - sv[u][k].y * tv[u].y,
                         sv[u][k].x * tv[u].y + sv[u][k].y * tv[u].x);
        }
    }
#pragma unroll 1
    for (; q < T; ++q) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const float2 tv = tab[(((q >> 1) * Ap + c0 + (uint32_t)k) << 1) + (q & 1u)];
            const float2 s = sp[k][0];
            sp[k] -= 1;
            add_pair(acc[k], s.x * tv.x - s.y * tv.y, s.x * tv.y + s.y * tv.x);
        }
    }
    float ar[R], ai[R];
#pragma unroll
    for (int k = 0; k < R; ++k) unpack_pair(acc[k], ar[k], ai[k]);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!act[k]) continue;
        const uint64_t phi = rx.nco_delta * j[k];
        const uint32_t idx = (rx.nco_log2 == 0) ? 0u : ((uint32_t)(phi >> 32) >> (32u - rx.nco_log2));
        const float2 rot = rx.nco[idx];
        rx.fine[(uint32_t)j[k] & rx.fine_mask] =
            make_float2(ar[k] * rot.x - ai[k] * rot.y, ar[k] * rot.y + ai[k] * rot.x);
    }
}

__global__ void __launch_bounds__(kTileThreads)
k_fine_tiles(const RxDev* __restrict__ rxs, const FineTile* __restrict__ tiles, uint32_t ntiles,
             const float2* __restrict__ chan, uint32_t* queue, const uint32_t* dyn) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ uint32_t s_it;
    __shared__ RxDev rx;
    if (dyn != nullptr) ntiles = *dyn;
    for (uint32_t u = next_tile(queue, &s_it); u < ntiles; u = next_tile(queue, &s_it)) {
        const FineTile t = tiles[u];
        if (threadIdx.x == 0) rx = rxs[t.rx];
        __syncthreads();
        const uint32_t T = rx.taps, Ap = rx.tile_cols, R = rx.tile_rows;
        float2* tab = sm;  // [ceil(T / 2)][Ap][2]: tap pairs
        float2* const buf0 = sm + ((T + 1u) >> 1) * 2u * Ap;
        float2* const buf1 = buf0 + kTileRows * rx.tile_stride;
        const uint32_t tid = threadIdx.x;
        const uint32_t n_a0 = t.a0 * rx.step_whole + (uint32_t)((uint64_t)t.a0 * rx.step_rem / rx.out_rate);
        // the table slice: taps q of columns [a0, a0 + width)
        {
            const uint32_t per = blockDim.x / t.width;
            const uint32_t c = tid % t.width;
            if (tid < per * t.width)
                for (uint32_t q = tid / t.width; q < T; q += per)
                    cp_async8(&tab[(((q >> 1) * Ap + c) << 1) + (q & 1u)],
                              &rx.lerped[(uint64_t)q * rx.period + (t.a0 + c) % rx.period]);
        }
        const uint32_t row = tid % kTileRows;
        const uint32_t c0 = (tid / kTileRows) * R;
        const bool computes = c0 < t.width;
        const uint32_t chunks = (t.rows + kTileRows - 1u) / kTileRows;
        stage_rows(buf0, rx, chan, t.row0, t.rows < kTileRows ? t.rows : kTileRows, n_a0);
        cp_async_commit();
        for (uint32_t ch = 0; ch < chunks; ++ch) {
            const uint32_t r0 = ch * kTileRows;
            const uint32_t nrows = (t.rows - r0) < kTileRows ? (t.rows - r0) : kTileRows;
            const float2* cur = (rx.tile_buffers == 2 && (ch & 1u)) ? buf1 : buf0;
            if (rx.tile_buffers == 2 && ch + 1u < chunks) {
                const uint32_t r1 = r0 + kTileRows;
                stage_rows((ch & 1u) ? buf0 : buf1, rx, chan, t.row0 + r1,
                           (t.rows - r1) < kTileRows ? (t.rows - r1) : kTileRows, n_a0);
                cp_async_commit();
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();  // table and this chunk staged by every thread
            if (computes) {
                if (R == 4)
                    compute_cols<4>(tab, cur, rx, t, t.row0 + r0, nrows, row, c0, n_a0);
                else if (R == 3)
                    compute_cols<3>(tab, cur, rx, t, t.row0 + r0, nrows, row, c0, n_a0);
                else if (R == 2)
                    compute_cols<2>(tab, cur, rx, t, t.row0 + r0, nrows, row, c0, n_a0);
                else
                    compute_cols<1>(tab, cur, rx, t, t.row0 + r0, nrows, row, c0, n_a0);
            }
            __syncthreads();  // everyone is done reading this chunk's buffer
            if (rx.tile_buffers != 2 && ch + 1u < chunks) {
                const uint32_t r1 = r0 + kTileRows;
                stage_rows(buf0, rx, chan, t.row0 + r1, (t.rows - r1) < kTileRows ? (t.rows - r1) : kTileRows, n_a0);
                cp_async_commit();
            }
        }
    }
}

}  // namespace

int32_t set_tile_shared(size_t shared) {
    cudaFuncAttributes attr;
    if (int32_t st = cuda_status(cudaFuncGetAttributes(&attr, (const void*)k_fine_tiles), "fine tiles attributes"))
        return st;
    if ((size_t)attr.maxDynamicSharedSizeBytes >= shared) return RV_OK;
    return cuda_status(cudaFuncSetAttribute((const void*)k_fine_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)shared),
                       "fine tiles shared memory");
}

int32_t launch_fine_tiles(cudaStream_t s, const RxDev* rxs, const FineTile* tiles, uint32_t ntiles,
                          const float2* chan, uint32_t shared_float2s, uint32_t* queue, const uint32_t* dyn) {
    if (ntiles == 0) return RV_OK;
    const size_t shared = (size_t)shared_float2s * sizeof(float2);
    if (int32_t st = set_tile_shared(shared)) return st;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (int32_t st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fine_tiles, kTileThreads, shared),
                                 "fine tiles occupancy"))
        return st;
    const int grid_cap = (per_sm > 0 ? per_sm : 1) * sms;
    const unsigned grid = dyn != nullptr ? (unsigned)grid_cap : (ntiles < (uint32_t)grid_cap ? ntiles : grid_cap);
    k_fine_tiles<<<grid, kTileThreads, shared, s>>>(rxs, tiles, ntiles, chan, queue, dyn);
    return cuda_status(cudaGetLastError(), "fine tiles");
}

}  // namespace rv
