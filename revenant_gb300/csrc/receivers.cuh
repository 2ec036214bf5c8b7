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
    uint32_t pad;
};

// A contiguous run of outputs of one receiver: fine outputs (fine stage),
// fine samples (detector stage) or audio frames (audio stage). `out` is where
// audio frames go in the run's audio buffer (in floats).
struct WorkItem {
    uint32_t rx;
    uint32_t count;
    uint64_t first;
    uint64_t out;
};

constexpr int kRxThreads = 256;

int32_t launch_lerp_table(cudaStream_t s, const rv_cf32* taps, float2* lerped, uint32_t T, uint32_t P,
                          uint32_t period, uint32_t step_rem, uint32_t fd, float inv_fd);
int32_t launch_fine_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                            const float2* chan, uint32_t window_cap);
int32_t launch_carrier_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems);
int32_t launch_detect_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                              uint32_t window_cap);
int32_t launch_audio_batched(cudaStream_t s, const RxDev* rxs, const WorkItem* items, uint32_t nitems,
                             float* audio, uint32_t window_cap);

}  // namespace rv
