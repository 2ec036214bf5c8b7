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
// Set-up: the device address of the array is looked up once per device
// context, on the first call made with that context current
// (cudaGetSymbolAddress; the host symbol itself is only a stand-in and must
// never reach a kernel). The lookups are kept by the context's unique id
// (cuCtxGetId, reached through cudaGetDriverEntryPointByVersion, so nothing
// links the driver library), so a context made after cudaDeviceReset or a
// different context on the same device gets its own lookup instead of a stale
// address. The first call in each context should therefore come before any
// stream capture is begun. Nothing here calls cudaMalloc, cudaFree or any
// allocating routine.
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
struct Lookup {
    unsigned long long context_id;
    rv_cf32* address;
};
Lookup g_scratch[kMaxDevices] = {};  // most recent contexts first
int g_lookups = 0;

using CtxGetCurrent = int (*)(void**);                    // cuCtxGetCurrent
using CtxGetId = int (*)(void*, unsigned long long*);     // cuCtxGetId
CtxGetCurrent g_get_current = nullptr;
CtxGetId g_get_id = nullptr;

// The unique id of the current context; *bound = false when this thread has
// none yet (the runtime binds it on its next call that needs the device).
int32_t current_context_id(unsigned long long* id, bool* bound) {
    if (g_get_current == nullptr || g_get_id == nullptr) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (int32_t st = rv::cuda_status(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa),
                                         "rv_pfb_channelize_noalloc: cuCtxGetCurrent"))
            return st;
        if (int32_t st = rv::cuda_status(cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb),
                                         "rv_pfb_channelize_noalloc: cuCtxGetId"))
            return st;
        if (qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || a == nullptr || b == nullptr)
            return rv::set_error_fmt(RV_ERR_UNSUPPORTED, "rv_pfb_channelize_noalloc: the driver lacks cuCtxGetId");
        g_get_current = reinterpret_cast<CtxGetCurrent>(a);
        g_get_id = reinterpret_cast<CtxGetId>(b);
    }
    void* ctx = nullptr;
    if (g_get_current(&ctx) != 0) return rv::set_error_fmt(RV_ERR_CUDA, "rv_pfb_channelize_noalloc: cuCtxGetCurrent failed");
    *bound = ctx != nullptr;
    if (ctx != nullptr && g_get_id(ctx, id) != 0)
        return rv::set_error_fmt(RV_ERR_CUDA, "rv_pfb_channelize_noalloc: cuCtxGetId failed");
    return RV_OK;
}

// Device address of the scratch array in the current context.
int32_t scratch_address(rv_cf32** out) {
    std::lock_guard<std::mutex> guard(g_lock);
    unsigned long long id = 0;
    bool bound = false;
    if (int32_t st = current_context_id(&id, &bound)) return st;
    if (bound)
        for (int i = 0; i < g_lookups; ++i)
            if (g_scratch[i].context_id == id) {
                *out = g_scratch[i].address;
                return RV_OK;
            }
    void* address = nullptr;
    if (int32_t st = rv::cuda_status(cudaGetSymbolAddress(&address, g_branch_scratch),
                                     "rv_pfb_channelize_noalloc: cudaGetSymbolAddress"))
        return st;
    if (!bound) {  // the lookup bound the runtime's context to this thread
        if (int32_t st = current_context_id(&id, &bound)) return st;
        if (!bound) return rv::set_error_fmt(RV_ERR_CUDA, "rv_pfb_channelize_noalloc: no current context");
        for (int i = 0; i < g_lookups; ++i)
            if (g_scratch[i].context_id == id) {
                *out = g_scratch[i].address;
                return RV_OK;
            }
    }
    // newest first; the oldest lookup drops out when the table is full
    const int keep = g_lookups < kMaxDevices ? g_lookups : kMaxDevices - 1;
    for (int i = keep; i > 0; --i) g_scratch[i] = g_scratch[i - 1];
    g_scratch[0] = Lookup{id, static_cast<rv_cf32*>(address)};
    g_lookups = keep + 1;
    *out = g_scratch[0].address;
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
