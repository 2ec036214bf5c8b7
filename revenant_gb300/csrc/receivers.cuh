// Device-side receiver table and work items shared by the batched receiver
// kernels (receivers.cu) and the chain runner (chain.cu).
#pragma once

#include <stdint.h>

#include "revenant_gb300.h"

namespace rv {

// One virtual receiver as the batched kernels see it: the fine stage's
// resampler and mixer constants (the per-receiver part of VrxFineParams),
// its tables, and the demodulator's configuration (VrxDemodConfig).
struct RxDev {
    // fine stage
    uint32_t chan_base;   // element offset of the receiver's channel in the channel ring
    uint32_t chan_mask;   // channel ring blocks - 1
    uint32_t taps;        // T
    uint32_t period;      // outputs after which the (phase, blend) pattern repeats
    uint32_t step_whole;  // channel_rate / demod_rate
    uint32_t step_rem;    // channel_rate % demod_rate
    uint32_t out_rate;    // demod_rate
    uint32_t nco_log2;
    uint64_t nco_delta;   // 0.64 turns per fine output
    const float2* lerped; // [period][T] taps already blended for each pattern phase, or null
    const float2* taps_raw;  // [P*T+1] polyphase table, used when lerped is null
    uint32_t phases;      // P
    float inv_out_rate;   // 1.0f / demod_rate, as resample_block computes it
    const float2* nco;    // shared NCO circle
    float2* fine;         // fine ring
    uint32_t fine_mask;
    // demodulator
    uint32_t mode, decimation, audio_taps, dc_taps, channels, pilot_taps;
    float gain;
    uint32_t reach;       // audio history in fine samples (fine history minus the detector's)
    const float* weights; // audio, dc, pilot pairs, rotation pairs
    float* det;           // detector output ring, one value per fine sample (same mask)
    uint32_t* carrier_state;  // 8 words, SAM / DSB only
    rv_vrx_carrier_params carrier;  // per-receiver loop constants
    uint32_t carrier_power;
    // fine stage as 2D tiles (fine_tiles.cu); tile_cols == 0: not tiled
    uint32_t tile_cols;     // columns of the table slice in shared memory (the block width)
    uint32_t tile_block;    // A: columns (pattern phases) per block
    uint32_t tile_rows;     // R: adjacent columns per thread (1 to 4)
    uint32_t tile_buffers;  // row chunks staged at once (2: the next chunk overlaps compute)
    uint32_t tile_seg;      // L: input samples of one row segment
    uint32_t tile_stride;   // float2 between row segments in shared memory (odd)
    uint32_t tile_period;   // P': outputs per row, a multiple of the pattern period
    uint32_t det_item;      // detector item: fine samples (batched detector)
    uint32_t audio_item;    // audio item: frames (batched audio)
    uint32_t tc_chunks;     // fast mode (fine_tc.cu): 64-element K chunks of each column group's GEMM
    uint64_t row_step;      // Dp = P' Fc / Fd: input samples between rows
    const uint16_t* tc_b;   // fast mode: the banded tap matrices, BF16 hi and lo, per group and chunk
};

// One receiver's detector and audio work of a run. The device splits it into
// items of det_item fine samples / audio_item frames: item k covers
// [first + k size, first + min(count, (k + 1) size)).
struct RxRun {
    uint64_t det_first;
    uint64_t audio_first;
    uint64_t audio_out;  // where the run's first frame goes in the audio buffer (floats)
    uint32_t det_count, audio_count;
};

// A run's item list of one stage: receiver r owns items [prefix[r],
// prefix[r + 1]); the host writes O(receivers) values, not one per item.
struct SpanList {
    const RxRun* runs;
    const uint32_t* prefix;  // [nrx + 1], exclusive prefix sums of item counts
    uint32_t nrx;
    uint32_t audio;          // 0: detector items, 1: audio items
};

// A contiguous run of outputs of one receiver: fine outputs (fine stage),
// fine samples (detector stage) or audio frames (audio stage). `out` is where
// audio frames go in the run's audio buffer (in floats), or the carrier's
// reset flag. Fine items carry the exact input index of their first output,
// its resampler fraction and pattern phase, computed on the host in 64 bits
// (resample_block, core/dsp/vrx_reference.cpp:2786-2810), and the length of
// the input window they stage.
struct WorkItem {
    uint32_t rx;
    uint32_t count;
    uint64_t first;
    uint64_t out;
    uint64_t n0;      // fine: input index of output `first`
    uint32_t frac0;   // fine: (first * (Fc mod Fd)) mod Fd
    uint32_t p0;      // fine: first mod period
    uint32_t window;  // fine: input samples staged (last input - n0 + T)
    uint32_t pad;
};

// A run of consecutive fine items of one receiver, processed by one CTA with
// the receiver's blended tap table in shared memory: `rows` tap rows
// ([rows][period] float2) at a time. rows == T keeps the whole table resident
// for the unit; rows < T passes the table through in row chunks for every
// item, each thread carrying its output's accumulator across chunks, so the
// per-output summation order (ascending tap) is unchanged.
struct FineUnit {
    uint32_t rx;
    uint32_t first_item;
    uint32_t items;
    uint32_t rows;
};

// Per-launch queue heads: items are handed out in list order, so the CTAs on
// an SM at any moment work on the same receiver (its tables stay in L1), and
// a slow item never holds up a fixed share of the list.
struct Queues {
    uint32_t fine, detect, audio, units, tiles, pad0, pad1, pad2;
};

// One tile of the 2D fine stage: columns [a0, a0 + width) of rows
// [row0, row0 + rows) of one receiver, where output j = row * P' + column;
// only outputs in [first, end), this run's, are written.
struct FineTile {
    uint32_t rx;
    uint32_t a0;
    uint32_t width;
    uint32_t rows;
    uint64_t row0;
    uint64_t first;
    uint64_t end;
};

// Fast mode's fine stage (fine_tc.cu): GEMM tiles of kFineTcRows rows by
// kFineTcColumns outputs; a FineTile then has a0 a multiple of the columns,
// width <= kFineTcColumns and rows <= kFineTcRows.
constexpr uint32_t kFineTcColumns = 32;
constexpr uint32_t kFineTcRows = 128;

constexpr int kTileThreads = 256;
constexpr uint32_t kTileRows = 16;  // rows per staged chunk: one half-warp
constexpr uint32_t kTileSlots = kTileThreads / kTileRows;  // column slots of R columns each

constexpr int kRxThreads = 256;

// Shared-memory layout of a mono audio FIR's weights: the taps, then four
// copies shifted by 1, 2, 3 and 4 taps, each 16-byte aligned and starting in a
// different bank quad, so that after a frame's first (partial) quad of
// samples every lane reads its weights as aligned four-tap vectors.
__host__ __device__ inline uint32_t mono_copy_base(uint32_t taps) { return (taps + 31u) & ~31u; }
__host__ __device__ inline uint32_t mono_copy_stride(uint32_t taps) { return ((taps + 3u + 31u) & ~31u) + 4u; }
// Stereo weights as the audio kernel stages them: per audio tap one float4
// {w[t], rotation[2t], rotation[2t + 1], 0}, then the pilot's (re, im) pairs.
__host__ __device__ inline uint32_t stereo_weight_floats(uint32_t taps, uint32_t pilot_taps) {
    return 4u * taps + 2u * pilot_taps;
}
__host__ __device__ inline uint32_t mono_weight_floats(uint32_t taps) {
    return mono_copy_base(taps) + 4u * mono_copy_stride(taps);
}

// The per-run values a captured run's kernels read from device memory
// instead of their launch arguments: the queue heads (zeroed by every
// upload), the item count of each list and the coarse kernel's parameters.
struct RunCounts {
    Queues queues;
    uint32_t units, fine, carrier, detect, audio, tiles, pad0, pad1;
    rv_coarse_params coarse;
    uint32_t pad2;
};

// Front-end correction in force for the raw samples a coarse launch reads
// (the fused kernel corrects samples as it converts them): entry k covers the
// samples from `rel_start` (relative to the launch's window start) up to the
// next entry's, `on` when the correction was applied to that run's samples.
constexpr uint32_t kFrontEndEntries = 16;
// The fused coarse kernel's input format for a cf32 sample ring that was
// converted, corrected and excised before it (impulse excision on).
constexpr int kFormatCf32Ring = 100;

struct FrontEndEntry {
    uint32_t rel_start, on;
    float dc_i, dc_q, cross, scale;
};
struct FrontEndTable {
    uint32_t count, pad;
    FrontEndEntry e[kFrontEndEntries];
};

// Every batched launcher takes `dyn`: nullptr for a direct launch, where
// `nitems` is the item count; or a device pointer to the count inside a
// RunCounts, for a launch captured in a CUDA graph, where `nitems` is the
// capacity of the list and the grid is the kernel's full resident grid.

int32_t launch_lerp_table(cudaStream_t s, const rv_cf32* taps, float2* lerped, uint32_t T, uint32_t P,
                          uint32_t period, uint32_t step_rem, uint32_t fd, float inv_fd);
int32_t launch_fine_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                            const float2* chan, uint32_t window_cap, uint32_t* queue, const uint32_t* dyn = nullptr);
// Units of fine items with shared-memory tap tables; `shared_floats2` is the
// dynamic shared memory per CTA (largest table + window), 1024 threads a CTA.
constexpr int kUnitThreads = 1024;
int32_t launch_fine_units(cudaStream_t s, const RxDev* rxs, const WorkItem* items, const FineUnit* units,
                          uint32_t nunits, const float2* chan, uint32_t shared_float2s, uint32_t* queue,
                          const uint32_t* dyn = nullptr);
uint32_t fine_unit_shared_budget();  // float2 entries of dynamic shared memory a CTA may use
// 2D tiles of the fine stage; `shared_float2s` of dynamic shared memory per
// CTA (the largest tiled receiver's table slice plus row buffers).
int32_t launch_fine_tiles(cudaStream_t s, const RxDev* rxs, const FineTile* tiles, uint32_t ntiles,
                          const float2* chan, uint32_t shared_float2s, uint32_t* queue, const uint32_t* dyn = nullptr);
// Fast mode: the chunks of a receiver's tables, their size in BF16 values,
// the table builder (from the blended taps) and the GEMM tiles' launch.
uint32_t fine_tc_chunks(uint32_t taps, uint32_t P, uint32_t step_whole, uint32_t step_rem, uint32_t fd);
uint64_t fine_tc_table_elements(uint32_t P, uint32_t chunks);
int32_t launch_fine_tc_tables(cudaStream_t s, const float2* lerped, uint32_t T, uint32_t period, uint32_t P,
                              uint32_t step_whole, uint32_t step_rem, uint32_t fd, uint32_t chunks, uint16_t* out);
int32_t launch_fine_tc(cudaStream_t s, const RxDev* rxs, const FineTile* tiles, uint32_t ntiles, const float2* chan,
                       uint32_t* queue, const uint32_t* dyn, uint32_t* status);
int32_t launch_carrier_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                               const uint32_t* dyn = nullptr);
// fast: fused multiply-adds in the DC-removal FIR (the chain's fast mode)
int32_t launch_detect_batched(cudaStream_t s, const RxDev* rxs, SpanList spans, uint32_t nitems,
                              uint32_t window_cap, uint32_t* queue, const uint32_t* dyn = nullptr, bool fast = false);
// weights_cap: floats of demodulator weights staged per CTA (the largest
// table among the receivers: audio taps, or the whole stereo table)
int32_t launch_audio_batched(cudaStream_t s, const RxDev* rxs, SpanList spans, uint32_t nitems,
                             float* audio, uint32_t window_cap, uint32_t weights_cap, uint32_t* queue,
                             const uint32_t* dyn = nullptr, bool fast = false);

}  // namespace rv
