// rv_pfb_channelize_noalloc: the branch filter and the FFT, with the branch
// values between them held in an array that lives inside this library.
//
// Who needs it: a caller that must not allocate device memory on its own
// path. A per-block processing callback cannot afford cudaMalloc there (the
// call can synchronise the whole device and take milliseconds while the
// stream behind it keeps arriving), and a plugin or host process that works
// inside someone else's fixed device-memory budget has no allocation rights
// at all. Such a caller still owns and passes every input and output; the only
// intermediate, the M values per block the branch filter hands to the FFT, is
// taken from a fixed file-scope device array instead of a buffer the caller
// would otherwise have to allocate.
//
// Limits and sharing: the array holds kNoAllocBranchValues complex values
// (8 MiB), so one call channelizes at most kNoAllocBranchValues / M blocks
// (16384 blocks at M = 64); larger requests are refused with RV_ERR_INVALID.
// Every GPU that loads the library keeps the array for the life of the
// process. All calls on a device share it and it keeps the last call's values:
// nothing in it needs to start at zero (the branch filter writes every value
// the FFT then reads), but two calls whose work overlaps on the GPU (different
// streams, no ordering between them) race on it.
//
// Set-up: the device address of the array is looked up once per device, on
// the first call made with that device current (cudaGetSymbolAddress; the host
// symbol itself is only a stand-in and must never reach a kernel). That first
// call should therefore come before any stream capture is begun. Nothing here
// calls cudaMalloc, cudaFree or any allocating routine.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "common.cuh"
#include "revenant_gb300.h"

namespace {

constexpr uint32_t kNoAllocBranchValues = RV_NOALLOC_BRANCH_VALUES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) rv_cf32 g_branch_scratch[kNoAllocBranchValues];

std::mutex g_lock;
rv_cf32* g_scratch[kMaxDevices] = {};

// Device address of the scratch array on the current device.
int32_t scratch_address(rv_cf32** out) {
    int device = 0;
    if (int32_t st = rv::cuda_status(cudaGetDevice(&device), "rv_pfb_channelize_noalloc: cudaGetDevice")) return st;
    if (device < 0 || device >= kMaxDevices)
        return rv::set_error_fmt(RV_ERR_UNSUPPORTED, "rv_pfb_channelize_noalloc: device %d", device);
    std::lock_guard<std::mutex> guard(g_lock);
    if (g_scratch[device] == nullptr) {
        void* address = nullptr;
        if (int32_t st = rv::cuda_status(cudaGetSymbolAddress(&address, g_branch_scratch),
                                         "rv_pfb_channelize_noalloc: cudaGetSymbolAddress"))
            return st;
        g_scratch[device] = static_cast<rv_cf32*>(address);
    }
    *out = g_scratch[device];
    return RV_OK;
}

}  // namespace

extern "C" int32_t rv_pfb_channelize_noalloc(void* stream, const rv_grid_params* grid,
                                             const rv_pfb_branch_params* branch_params,
                                             const rv_pfb_fft_params* fft_params, const float* taps_dev,
                                             uint64_t taps_len, const rv_cf32* ring_dev, uint64_t ring_len,
                                             const rv_cf32* twiddles_dev, uint64_t twiddles_len,
                                             rv_cf32* channel_ring_dev, uint64_t channel_ring_len) {
    if (grid == nullptr || branch_params == nullptr || fft_params == nullptr)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_pfb_channelize_noalloc: NULL argument");
    if (fft_params->channels != grid->channels || fft_params->decimation != grid->decimation)
        return rv::set_error_fmt(RV_ERR_INVALID,
                                 "rv_pfb_channelize_noalloc: the FFT's M=%u D=%u differ from the grid's M=%u D=%u",
                                 fft_params->channels, fft_params->decimation, grid->channels, grid->decimation);
    if (fft_params->block_count != branch_params->block_count)
        return rv::set_error_fmt(RV_ERR_INVALID,
                                 "rv_pfb_channelize_noalloc: the branch filter makes %u blocks and the FFT reads %u",
                                 branch_params->block_count, fft_params->block_count);
    const uint64_t values = (uint64_t)branch_params->block_count * grid->channels;
    if (values > kNoAllocBranchValues)
        return rv::set_error_fmt(RV_ERR_INVALID,
                                 "rv_pfb_channelize_noalloc: %u blocks of %u channels need %llu branch values; the "
                                 "library's fixed scratch holds %u (at most %u blocks at this M)",
                                 branch_params->block_count, grid->channels, (unsigned long long)values,
                                 kNoAllocBranchValues, kNoAllocBranchValues / grid->channels);
    rv_cf32* scratch = nullptr;
    if (int32_t st = scratch_address(&scratch)) return st;
    if (int32_t st = rv_pfb_branch(stream, grid, branch_params, taps_dev, taps_len, ring_dev, ring_len, scratch,
                                   kNoAllocBranchValues))
        return st;
    return rv_pfb_fft(stream, fft_params, scratch, kNoAllocBranchValues, twiddles_dev, twiddles_len, channel_ring_dev,
                      channel_ring_len);
}
