// The learned proposal's spectrogram tiles and its proposed bin ranges.
//
// Tiles. A row of tiles covers RV_TILE_FRAMES consecutive spectrum frames
// (dB, the detector's input) and every bin; tile t holds bins
// [256 t, 256 t + 256). Two channels per pixel, each the dB of an
// exponential average of the linear power, frame by frame:
//   0: with a tenth of the detector's time constant (a burst shows there as
//      it starts and stops)
//   1: with the detector's time constant (the detector decides on such an
//      average, so a burst that ended a second ago still shows there)
// Both less the row's noise floor (the median over the row's tiles of each
// tile's mean channel-1 dB), divided by 10 and rounded to BF16.
//
//   k_tile_average   one thread per bin: the average over the row's frames,
//                    both channels into an FP32 staging row in tile order,
//                    and per tile the mean of channel 1 (one block per tile)
//   k_tile_floor     one block: the median of the tile means (bitonic sort)
//   k_tile_pack      the staging row less the floor, / 10, to BF16
//
// Regions. A cell (8 bins of a tile) is proposed when its logit is above the
// threshold; the cells' flags come back to the host, are held for hold_rows
// further rows and merged into padded bin ranges.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "common.cuh"

namespace rv {
namespace {

constexpr uint32_t kTileFrames = RV_TILE_FRAMES;
constexpr uint32_t kTileBins = RV_TILE_BINS;
constexpr uint32_t kCells = RV_CNN_CELLS;
constexpr float kDbToLog2 = 0.332192809488736234787F;  // log2(10) / 10

// One block of 256 threads per tile: bin = 256 t + thread.
__global__ void __launch_bounds__(256) k_tile_average(const float* __restrict__ frames, uint32_t bins, float alpha,
                                                      float alpha_short, uint32_t fresh, float* __restrict__ average,
                                                      float* __restrict__ staging, float* __restrict__ tile_mean) {
    const uint32_t t = blockIdx.x, b = threadIdx.x, bin = t * kTileBins + b;
    float a = average[bin], q = average[bins + bin];
    float sum = 0.0F;
    float* out = staging + (uint64_t)t * kTileFrames * kTileBins * 2u;
    for (uint32_t f = 0; f < kTileFrames; ++f) {
        const float db = frames[(uint64_t)f * bins + bin];
        const float linear = exp2f(db * kDbToLog2);
        a = (fresh && f == 0) ? linear : a + alpha * (linear - a);
        q = (fresh && f == 0) ? linear : q + alpha_short * (linear - q);
        const float adb = 10.0F * log10f(fmaxf(a, 1.0e-30F));
        const float qdb = 10.0F * log10f(fmaxf(q, 1.0e-30F));
        *reinterpret_cast<float2*>(out + ((uint64_t)f * kTileBins + b) * 2u) = make_float2(qdb, adb);
        sum += adb;
    }
    average[bin] = a;
    average[bins + bin] = q;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
    __shared__ float part[8];
    if ((b & 31u) == 0) part[b >> 5] = sum;
    __syncthreads();
    if (b == 0) {
        float s = 0.0F;
        for (int w = 0; w < 8; ++w) s += part[w];
        tile_mean[t] = s / (float)(kTileFrames * kTileBins);
    }
}

// One block of 1024 threads: the median of `tiles` values (<= 1024).
__global__ void __launch_bounds__(1024) k_tile_floor(const float* __restrict__ tile_mean, uint32_t tiles,
                                                     float* __restrict__ floor_db) {
    __shared__ float v[1024];
    const uint32_t i = threadIdx.x;
    v[i] = i < tiles ? tile_mean[i] : INFINITY;
    __syncthreads();
    for (uint32_t k = 2; k <= 1024u; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            const uint32_t p = i ^ j;
            if (p > i) {
                const bool up = (i & k) == 0;
                const float x = v[i], y = v[p];
                if ((x > y) == up) {
                    v[i] = y;
                    v[p] = x;
                }
            }
            __syncthreads();
        }
    if (i == 0) *floor_db = v[(tiles - 1u) / 2u];
}

__global__ void k_tile_pack(const float* __restrict__ staging, uint64_t pairs, const float* __restrict__ floor_db,
                            __nv_bfloat162* __restrict__ tiles) {
    const float f = *floor_db;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < pairs; i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 x = reinterpret_cast<const float2*>(staging)[i];
        tiles[i] = __floats2bfloat162_rn((x.x - f) * 0.1F, (x.y - f) * 0.1F);
    }
}

__global__ void k_cell_flags(const float* __restrict__ logits, uint32_t n, float threshold, uint8_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = logits[i] > threshold ? 1u : 0u;
}

}  // namespace
}  // namespace rv

using namespace rv;

struct rv_proposer {
    rv_context* context = nullptr;
    cudaStream_t stream = nullptr;
    rv_proposal_config config{};
    uint32_t tiles = 0;
    float alpha = 0.0F, alpha_short = 0.0F;
    bool fresh = true;
    float* average = nullptr;   // bins (long) then bins (short)
    float* staging = nullptr;   // one tile row, FP32
    float* tile_mean = nullptr; // tiles
    float* floor_db = nullptr;  // 1
    uint8_t* flags = nullptr;   // tiles * cells
    uint8_t* flags_host = nullptr;
    std::vector<std::vector<uint8_t>> held;  // the last hold_rows rows' flags, newest last
};

extern "C" {

int32_t rv_proposer_create(rv_context* context, const rv_proposal_config* c, rv_proposer** out) {
    if (context == nullptr || c == nullptr || out == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_create: NULL argument");
    *out = nullptr;
    if (c->bins == 0 || c->bins % kTileBins != 0 || c->bins / kTileBins > 1024u)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_create: %u bins (a multiple of %u, at most %u)", c->bins,
                             kTileBins, 1024u * kTileBins);
    if (!(c->frame_seconds > 0.0) || !(c->average_seconds > 0.0) || !std::isfinite(c->frame_seconds) ||
        !std::isfinite(c->average_seconds))
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_create: frame_seconds %g, average_seconds %g", c->frame_seconds,
                             c->average_seconds);
    if (c->hold_rows > 64u) return set_error_fmt(RV_ERR_INVALID, "rv_proposer_create: hold_rows %u (at most 64)", c->hold_rows);
    rv_proposer* p = new (std::nothrow) rv_proposer;
    if (p == nullptr) return set_error_fmt(RV_ERR_NO_MEMORY, "rv_proposer_create: out of host memory");
    p->context = context;
    p->stream = reinterpret_cast<cudaStream_t>(rv_context_stream(context));
    p->config = *c;
    p->tiles = c->bins / kTileBins;
    p->alpha = (float)std::min(1.0, std::max(1.0e-6, 1.0 - std::exp(-c->frame_seconds / c->average_seconds)));
    p->alpha_short = (float)std::min(1.0, std::max(1.0e-6, 1.0 - std::exp(-10.0 * c->frame_seconds / c->average_seconds)));
    const uint64_t staging = (uint64_t)c->bins * kTileFrames * 2u;
    int32_t st = cuda_status(cudaMalloc(&p->average, 2u * c->bins * sizeof(float)), "proposer allocation");
    if (!st) st = cuda_status(cudaMalloc(&p->staging, staging * sizeof(float)), "proposer allocation");
    if (!st) st = cuda_status(cudaMalloc(&p->tile_mean, p->tiles * sizeof(float)), "proposer allocation");
    if (!st) st = cuda_status(cudaMalloc(&p->floor_db, sizeof(float)), "proposer allocation");
    if (!st) st = cuda_status(cudaMalloc(&p->flags, (size_t)p->tiles * kCells), "proposer allocation");
    if (!st) st = cuda_status(cudaHostAlloc(&p->flags_host, (size_t)p->tiles * kCells, cudaHostAllocDefault),
                              "proposer allocation");
    if (st) {
        rv_proposer_destroy(p);
        return st;
    }
    *out = p;
    return clear_error();
}

int32_t rv_proposer_destroy(rv_proposer* p) {
    if (p == nullptr) return RV_OK;
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (void* q : {(void*)p->average, (void*)p->staging, (void*)p->tile_mean, (void*)p->floor_db, (void*)p->flags})
        if (q) cudaFree(q);
    if (p->flags_host) cudaFreeHost(p->flags_host);
    delete p;
    return clear_error();
}

int32_t rv_proposer_set_stream(rv_proposer* p, void* stream) {
    if (p == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_proposer_set_stream: NULL");
    if (int32_t st = cuda_status(cudaStreamSynchronize(p->stream), "proposer stream")) return st;
    p->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : reinterpret_cast<cudaStream_t>(rv_context_stream(p->context));
    return clear_error();
}

int32_t rv_proposer_reset(rv_proposer* p) {
    if (p == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_proposer_reset: NULL");
    p->fresh = true;
    p->held.clear();
    return clear_error();
}

int32_t rv_proposer_tiles(rv_proposer* p, const float* frames_dev, uint64_t frames_len, void* tiles_dev,
                          uint64_t tiles_len) {
    if (p == nullptr || frames_dev == nullptr || tiles_dev == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_tiles: NULL argument");
    const uint64_t need_frames = (uint64_t)kTileFrames * p->config.bins;
    const uint64_t need_tiles = (uint64_t)p->config.bins * kTileFrames * 2u;  // BF16 values
    if (frames_len < need_frames)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_tiles: %llu frame values for %llu",
                             (unsigned long long)frames_len, (unsigned long long)need_frames);
    if (tiles_len < need_tiles)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_tiles: room for %llu tile values, %llu needed",
                             (unsigned long long)tiles_len, (unsigned long long)need_tiles);
    if ((reinterpret_cast<uintptr_t>(tiles_dev) & 15u) != 0)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_tiles: tiles must be 16-byte aligned");
    k_tile_average<<<p->tiles, kTileBins, 0, p->stream>>>(frames_dev, p->config.bins, p->alpha, p->alpha_short,
                                                          p->fresh ? 1u : 0u, p->average, p->staging, p->tile_mean);
    if (int32_t st = cuda_status(cudaGetLastError(), "tile average")) return st;
    k_tile_floor<<<1, 1024, 0, p->stream>>>(p->tile_mean, p->tiles, p->floor_db);
    if (int32_t st = cuda_status(cudaGetLastError(), "tile floor")) return st;
    const uint64_t pairs = need_tiles / 2u;
    k_tile_pack<<<(uint32_t)std::min<uint64_t>((pairs + 255u) / 256u, 8192u), 256, 0, p->stream>>>(
        p->staging, pairs, p->floor_db, reinterpret_cast<__nv_bfloat162*>(tiles_dev));
    if (int32_t st = cuda_status(cudaGetLastError(), "tile pack")) return st;
    p->fresh = false;
    return clear_error();
}

int32_t rv_proposer_regions(rv_proposer* p, const float* logits_dev, uint64_t logits_len, uint32_t* ranges,
                            uint32_t capacity, uint32_t* count) {
    if (p == nullptr || logits_dev == nullptr || count == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_regions: NULL argument");
    const uint32_t cells = p->tiles * kCells;
    if (logits_len < cells)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_regions: %llu logits for %u cells", (unsigned long long)logits_len,
                             cells);
    k_cell_flags<<<(cells + 255u) / 256u, 256, 0, p->stream>>>(logits_dev, cells, p->config.threshold, p->flags);
    if (int32_t st = cuda_status(cudaGetLastError(), "proposal flags")) return st;
    if (int32_t st = cuda_status(cudaMemcpyAsync(p->flags_host, p->flags, cells, cudaMemcpyDeviceToHost, p->stream),
                                 "proposal flags"))
        return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(p->stream), "proposal flags")) return st;
    p->held.emplace_back(p->flags_host, p->flags_host + cells);
    while (p->held.size() > (size_t)p->config.hold_rows + 1u) p->held.erase(p->held.begin());
    // runs of proposed cells (in any held row), padded and merged
    const uint32_t bins = p->config.bins, pad = p->config.pad_bins;
    uint32_t n = 0;
    uint32_t cur_lo = 0, cur_hi = 0;
    bool open = false;
    auto flush = [&]() {
        if (!open) return;
        if (ranges != nullptr && n < capacity) {
            ranges[2u * n] = cur_lo;
            ranges[2u * n + 1u] = cur_hi;
        }
        ++n;
        open = false;
    };
    for (uint32_t c = 0; c < cells; ++c) {
        bool on = false;
        for (const auto& row : p->held) on = on || row[c] != 0;
        if (!on) continue;
        const uint32_t lo = c * RV_CNN_CELL_BINS > pad ? c * RV_CNN_CELL_BINS - pad : 0u;
        const uint32_t hi = std::min(bins, (c + 1u) * RV_CNN_CELL_BINS + pad);
        if (open && lo <= cur_hi) {
            cur_hi = std::max(cur_hi, hi);
        } else {
            flush();
            cur_lo = lo;
            cur_hi = hi;
            open = true;
        }
    }
    flush();
    *count = n;
    if (ranges != nullptr && n > capacity)
        return set_error_fmt(RV_ERR_INVALID, "rv_proposer_regions: %u ranges for room of %u", n, capacity);
    return clear_error();
}

}  // extern "C"
