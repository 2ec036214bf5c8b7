// The receive chain: raw IQ in, channel ring, N virtual receivers, audio out.
//
// Host-side equivalent of Graph::on_block + DemodStage::record
// (core/engine/graph.cpp:4770-5485, core/engine/vrx_stage.cpp:1119-1430): per
// run of input samples it converts and channelizes the new blocks, then
// advances every receiver's fine stage, carrier loop and demodulator by
// exactly the outputs whose inputs now exist, with the reference's cursor
// arithmetic (highest_output_for / lowest_output_for, anchor_to).
//
// Two execution modes share that bookkeeping and produce identical bits:
//  * RV_CHAIN_PLAIN: the reference's recording, one launch per stage per
//    receiver (convert, branch, FFT, then fine [+ carrier] + demod for each
//    receiver) through the plain kernels. This is the baseline.
//  * RV_CHAIN_BATCHED: the fused coarse kernel, then one launch per receiver
//    stage covering every receiver (fine, carrier, detector, audio), driven by
//    work lists built on the host and uploaded once per run.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <new>
#include <numeric>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "receivers.cuh"
#include "revenant_gb300.h"

namespace rv {
int32_t plan_receiver(const rv_grid_params& g, int64_t rate, const rv_vrx_request& r, rv_vrx_plan_info& info,
                      std::vector<rv_cf32>& taps, std::vector<float>& weights);
int32_t design_prototype_table(const rv_grid_params& g, double atten, std::vector<float>& taps);
int32_t build_twiddle_table(uint32_t M, std::vector<rv_cf32>& out);
int32_t build_nco(uint32_t log2, std::vector<rv_cf32>& out);
int32_t validate_grid(const rv_grid_params* g);
uint32_t demod_fine_history(const rv_vrx_demod_config* c);
int32_t launch_iq_moments(cudaStream_t s, const rv_iq_moments_params& p, const rv_cf32* ring, float* sums);
int32_t launch_iq_moments_raw(cudaStream_t s, int32_t format, const rv_iq_moments_params& p, const void* raw,
                              float* sums);
void front_end_update(rv_front_end* st, const double totals[5], uint64_t samples, int64_t rate);
void total_moments(const float* sums, uint64_t chunks, double totals[5]);
int32_t build_window(uint32_t n, uint32_t t, double a, std::vector<float>& out);
int32_t detector_wait_for(rv_detector* d, cudaStream_t producer);
int32_t detector_release_to(rv_detector* d, cudaStream_t producer);
int32_t launch_coarse_fused(cudaStream_t stream, const rv_grid_params& g, int32_t format, const rv_coarse_params& p,
                            const void* raw, const float* taps, const rv_cf32* tw, rv_cf32* ring,
                            const rv_coarse_params* dyn = nullptr, const FrontEndTable* fe = nullptr);
int32_t launch_convert_ring(cudaStream_t stream, int32_t format, const void* raw, uint32_t mask, uint32_t from,
                            uint32_t count, uint32_t window_start, const FrontEndTable* fe, rv_cf32* clean);
bool coarse_fused_supported(const rv_grid_params& g);
}  // namespace rv

using namespace rv;

namespace {

constexpr uint32_t kFineWindow = 6144;   // float2 per fine work item (48 KB)
constexpr uint32_t kDetWindow = 8192;    // floats per detector / audio item (32 KB)
constexpr uint32_t kMaxItem = kRxThreads;
constexpr uint64_t kMaxLerpEntries = 1u << 20;
constexpr uint32_t kTileShare = 2;  // fine tiles aim at this many CTAs per SM

uint64_t bit_ceil64(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

// core/engine/vrx_stage.cpp:173-197
uint64_t highest_output_for(uint64_t newest, uint64_t fc, uint64_t fd) {
    const uint64_t bound = newest + 1u, whole = bound / fc, part = bound % fc;
    if (part == 0) return whole * fd - 1u;
    return whole * fd + (part * fd - 1u) / fc;
}
uint64_t lowest_output_for(uint64_t needed, uint64_t fc, uint64_t fd) {
    const uint64_t whole = needed / fc, part = needed % fc;
    return whole * fd + (part * fd + fc - 1u) / fc;
}

template <class T>
struct DeviceArray {
    T* ptr = nullptr;
    size_t count = 0;
    int32_t alloc(size_t n) {
        release();
        if (n == 0) n = 1;
        if (int32_t st = cuda_status(cudaMalloc(&ptr, n * sizeof(T)), "chain allocation")) return st;
        count = n;
        return RV_OK;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
};

template <class T>
struct PinnedArray {
    T* ptr = nullptr;
    size_t count = 0;
    int32_t reserve(size_t n) {
        if (n <= count) return RV_OK;
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        count = 0;
        if (int32_t st = cuda_status(cudaHostAlloc(&ptr, n * sizeof(T), cudaHostAllocDefault), "chain pinned"))
            return st;
        count = n;
        return RV_OK;
    }
    void release() {
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        count = 0;
    }
};

struct Receiver {
    rv_vrx_request request{};
    rv_vrx_plan_info plan{};
    std::vector<rv_cf32> taps;
    std::vector<float> weights;
    uint32_t period = 0;
    uint32_t fine_history = 0, det_history = 0, reach = 0;
    uint32_t fine_mask = 0;
    uint32_t max_fine_item = 0, max_det_item = 0, max_audio_item = 0;
    uint32_t table_rows = 0;      // tap rows of the blended table staged at a time by the unit kernel
    uint32_t max_unit_item = 0;   // outputs per item on the unit path
    // 2D tiles (fine_tiles.cu); tile_cols == 0: the unit or per-item path
    uint32_t tile_cols = 0, tile_block = 0, tile_rows = 0, tile_buffers = 0, tile_seg = 0, tile_stride = 0;
    uint32_t tile_period = 0;
    uint64_t row_step = 0;
    uint32_t tile_shared = 0;     // float2 of shared memory a tile of this receiver needs
    uint32_t tc_chunks = 0;       // fast mode: K chunks of its GEMM tiles (0: the exact tiles)
    DeviceArray<uint16_t> d_tc;   // fast mode: banded tap matrices (fine_tc.cu)
    bool started = false;
    bool carrier_reset = true;
    uint64_t first_output = 0, next_output = 0, next_audio = 0;
    uint64_t audio_frames_total = 0;
    DeviceArray<rv_cf32> d_taps;
    DeviceArray<float2> d_lerped;
    DeviceArray<rv_cf32> d_fine;
    DeviceArray<float> d_det;
    DeviceArray<float> d_weights;
    DeviceArray<uint32_t> d_state;
    std::vector<float> audio;  // accumulated on the host when keep_audio
    uint64_t run_audio_offset = 0, run_audio_frames = 0;
};

// What a captured graph was built for: the capacity of each work list (its
// section of the device item array), the launch shapes and the buffers baked
// into its kernel arguments. A run that needs more, or different buffers,
// captures again.
struct GraphShape {
    uint32_t fine = 0, carrier = 0, unit_items = 0, units = 0, tiles = 0, nrx = 0;
    uint32_t fine_window = 0, weights_cap = 0, unit_budget = 0, tile_shared = 0, front_end = 0, excision = 0;
    const void* tiles_ptr = nullptr;
    const void* spans_ptr = nullptr;
    const void* audio_ptr = nullptr;
    const void* table_ptr = nullptr;
    const void* items_ptr = nullptr;
    const void* units_ptr = nullptr;
};

// The buffers one run's launches read and write, its captured graph and its
// audio on the way to the host. A pipelined chain alternates two, so that one
// run is prepared and its input copied while the previous one executes.
struct RunSlot {
    PinnedArray<WorkItem> items_host;
    DeviceArray<WorkItem> items_dev;
    DeviceArray<Queues> queues;
    DeviceArray<FineUnit> units_dev;
    PinnedArray<FineUnit> units_host;
    DeviceArray<FineTile> tiles_dev;
    PinnedArray<FineTile> tiles_host;
    DeviceArray<uint8_t> spans_dev;   // RxRun[nrx], detector prefix [nrx + 1], audio prefix [nrx + 1]
    PinnedArray<uint8_t> spans_host;
    DeviceArray<float> audio_dev;
    PinnedArray<float> audio_host;
    cudaGraphExec_t exec = nullptr;
    GraphShape shape{};
    DeviceArray<RunCounts> counts_dev;
    PinnedArray<RunCounts> counts_host;
    cudaEvent_t done = nullptr;  // recorded after the run's audio read-back
    bool pending = false;        // audio not yet handed to the receivers
    // front-end moments of the run, read back with its audio
    DeviceArray<float> sums_dev;
    PinnedArray<float> sums_host;
    DeviceArray<FrontEndTable> fe_dev;
    PinnedArray<FrontEndTable> fe_host;
    uint32_t sums_count = 0;
    uint64_t sums_run = 0;
    bool sums_pending = false;
    uint64_t audio_floats = 0;
    std::vector<std::pair<uint64_t, uint64_t>> parts;  // per receiver: audio offset (floats), frames
    void release() {
        items_host.release();
        items_dev.release();
        queues.release();
        units_dev.release();
        units_host.release();
        tiles_dev.release();
        tiles_host.release();
        spans_dev.release();
        spans_host.release();
        audio_dev.release();
        audio_host.release();
        counts_dev.release();
        counts_host.release();
        sums_dev.release();
        sums_host.release();
        fe_dev.release();
        fe_host.release();
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (done) cudaEventDestroy(done);
        done = nullptr;
    }
};

}  // namespace

struct rv_chain {
    rv_context* context = nullptr;
    cudaStream_t stream = nullptr;
    rv_chain_config config{};
    bool fast = false;                 // RV_CHAIN_FAST: a batched chain with the fine stage on the tensor cores
    bool hoisted = false;              // RV_CHAIN_HOISTED: a batched chain whose receiver stages launch per receiver
    uint32_t tiles_per_sm = 4;         // fine tiles a run is cut into, per SM (rv_chain_autotune may change it)
    DeviceArray<uint32_t> hoisted_prefix;  // per receiver: its detector then audio item prefix sums
    DeviceArray<uint32_t> tc_status;   // fast mode: tensor-core waits that ran out
    uint32_t stages = 0;
    uint32_t bytes_per_sample = 0;
    // rings
    uint32_t raw_mask = 0;         // raw ring capacity (samples) - 1
    uint32_t chan_blocks = 0;      // channel ring blocks per channel
    DeviceArray<uint8_t> raw;      // batched: native-format ring; plain: staging for one run
    DeviceArray<rv_cf32> cf32_ring;  // plain only
    DeviceArray<rv_cf32> branch;     // plain only
    DeviceArray<rv_cf32> channel;
    DeviceArray<float> proto;
    DeviceArray<rv_cf32> twiddles;
    DeviceArray<rv_cf32> nco;
    std::vector<float> proto_host;
    std::vector<Receiver> rx;
    DeviceArray<RxDev> rx_table;
    bool table_dirty = true;
    // per-run buffers: slot 0 only, or both alternately when pipelined
    RunSlot slots[2];
    uint32_t cur = 0;
    cudaStream_t copy_stream = nullptr;  // pipelined: input copies
    cudaEvent_t input_ready = nullptr;
    uint32_t unit_budget = 0;
    uint32_t tile_shared = 0;   // float2 of shared memory per tile CTA (largest tiled receiver)
    uint32_t weights_cap = 32;  // largest staged demodulator weight table (floats)
    uint64_t samples_in = 0;
    uint64_t next_block = 0;
    rv_chain_stats stats{};
    // stage boundaries for profiling: input, coarse, fine, demod, readback
    cudaEvent_t marks[6] = {};
    // captured runs (rv_chain_capture_graph)
    bool graph = false;
    bool captured_run = false;  // this run replayed the graph
    // front-end correction (Graph::set_front_end_correction)
    bool fe_dc = false, fe_iq = false, fe_was_on = false;
    uint32_t fe_lag = 1;
    rv_front_end fe{};
    uint64_t run_index = 0;
    struct FePending {
        uint64_t run;
        uint32_t count;
        double totals[5];
    };
    std::vector<FePending> fe_pending;  // moments not yet in the estimate
    struct FeRun {
        uint64_t start, end;  // the run's source samples
        FrontEndEntry entry;  // the correction applied to them
    };
    std::vector<FeRun> fe_runs;  // the runs a coarse window can still reach
    const FrontEndTable* fe_table = nullptr;  // this run's table on the device, or none
    // spectrum stage (Graph::on_block's spectrum dispatch) and its consumer
    uint32_t spec_n = 0;  // transform points per channel; 0 = off
    DeviceArray<float> spec_window;
    DeviceArray<rv_cf32> spec_twiddles;
    DeviceArray<float> spec_frame;
    uint64_t spec_start = 0, spec_count = 0, spec_sequence = 0;
    bool spec_recorded = false;
    uint64_t group_delay = 0;  // the prototype's, in input samples
    rv_detector* detector = nullptr;
    // impulse excision (Graph::plan_impulse_excision / record_impulse_excision)
    bool ex_on = false, ex_was_on = false;
    rv_excision_config ex_cfg{};
    rv_excision_rings ex_rings{};
    rv_excision_cursor ex_cursor{};
    float ex_threshold = 0.0F;
    DeviceArray<rv_cf32> clean;  // batched: the converted, corrected, excised samples (raw ring's slots)
    DeviceArray<float> ex_seg_power, ex_seg_level;
    DeviceArray<uint32_t> ex_flags, ex_counters;
    DeviceArray<rv_cf32> ex_removed;
    rv_excision_plan ex_plan{};
    uint64_t ex_converted_end = 0;  // batched: the clean ring holds converted samples up to here
    // batched: the channelizer reads the clean ring. Set once the stage was
    // on, and kept after it is switched off, because the channelizer's history
    // still reaches back into samples the stage excised.
    bool ex_clean = false;
    // batched: a fused coarse kernel exists for the grid; otherwise the
    // channelizer runs as the plain branch and FFT dispatches over the clean
    // ring, and the receivers stay batched
    bool fused = true;
    uint64_t ex_examined = 0;
    uint64_t ex_totals[3] = {0, 0, 0};  // samples, events, spared read back so far
};

namespace {
RunSlot& S(rv_chain* c) { return c->slots[c->cur]; }
bool pipelined(const rv_chain* c) { return c->config.pipelined != 0; }
}  // namespace

namespace {
void mark(rv_chain* c, int i) {
    if (c->config.profile && !pipelined(c) && c->marks[i]) cudaEventRecord(c->marks[i], c->stream);
}
void collect_marks(rv_chain* c) {
    if (!c->config.profile || pipelined(c)) return;
    float ms[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&ms[i], c->marks[i], c->marks[i + 1]);
    c->stats.input_ms += ms[0];
    if (c->captured_run) {
        // the graph's stages are not separable: work-list upload + graph
        c->stats.graph_ms += ms[1] + ms[2] + ms[3];
    } else {
        c->stats.coarse_ms += ms[1];
        c->stats.fine_ms += ms[2];
        c->stats.demod_ms += ms[3];
    }
    c->stats.readback_ms += ms[4];
}
}  // namespace

namespace {

// Hands a finished run's audio to its receivers (waits for the run first).
// A finished run's front-end moments, totalled in chunk order, into the
// estimator's queue (core/dsp/front_end_correction.cpp total_moments).
void fe_collect(rv_chain* c, RunSlot& sl) {
    if (!sl.sums_pending) return;
    sl.sums_pending = false;
    rv_chain::FePending p{sl.sums_run, sl.sums_count, {0, 0, 0, 0, 0}};
    total_moments(sl.sums_host.ptr, (sl.sums_count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK, p.totals);
    c->fe_pending.push_back(p);
}

int32_t collect_slot(rv_chain* c, RunSlot& sl) {
    if (!sl.pending) return RV_OK;
    if (int32_t st = cuda_status(cudaEventSynchronize(sl.done), "run completion")) return st;
    sl.pending = false;
    fe_collect(c, sl);
    for (size_t i = 0; i < sl.parts.size() && i < c->rx.size(); ++i) {
        Receiver& r = c->rx[i];
        const uint64_t frames = sl.parts[i].second, n = frames * r.plan.demod.channels;
        if (c->config.keep_audio && n)
            r.audio.insert(r.audio.end(), sl.audio_host.ptr + sl.parts[i].first, sl.audio_host.ptr + sl.parts[i].first + n);
        r.audio_frames_total += frames;
    }
    c->stats.audio_bytes += sl.audio_floats * sizeof(float);
    return RV_OK;
}

// Every run still in flight, oldest first (the current slot holds the older
// one after a pipelined run flipped it).
int32_t collect_all(rv_chain* c) {
    if (int32_t st = collect_slot(c, c->slots[c->cur])) return st;
    return collect_slot(c, c->slots[c->cur ^ 1u]);
}

// Graph::record_front_end_correction's bookkeeping (core/engine/graph.cpp:
// 1382-1436) for the run of `count` samples from `first_sample`: reset when
// switched on, the estimate brought up to the runs `fe_lag` or more before
// this one (the engine's estimate lags by its frames in flight), and the
// correction this run's samples get, remembered for later coarse windows.
FrontEndEntry fe_prepare(rv_chain* c, uint64_t first_sample, uint64_t count, bool* on) {
    *on = c->fe_dc || c->fe_iq;
    if (*on && !c->fe_was_on) {
        rv_front_end_reset(&c->fe);
        c->fe_pending.clear();
    }
    c->fe_was_on = *on;
    size_t used = 0;
    for (; used < c->fe_pending.size() && c->fe_pending[used].run + c->fe_lag <= c->run_index; ++used)
        front_end_update(&c->fe, c->fe_pending[used].totals, c->fe_pending[used].count, c->config.rate);
    c->fe_pending.erase(c->fe_pending.begin(), c->fe_pending.begin() + (ptrdiff_t)used);
    FrontEndEntry e{0u, 0u, 0.0F, 0.0F, 0.0F, 1.0F};
    if (*on && count > 0 && c->fe.measured) {
        rv_iq_correct_params cp;
        rv_front_end_correction(&c->fe, c->fe_dc ? 1 : 0, c->fe_iq ? 1 : 0, &cp);
        e = FrontEndEntry{0u, 1u, cp.dc_i, cp.dc_q, cp.cross, cp.scale};
    }
    c->fe_runs.push_back(rv_chain::FeRun{first_sample, first_sample + count, e});
    if (c->fe_runs.size() > 4u * kFrontEndEntries)  // a plain chain never reads them back
        c->fe_runs.erase(c->fe_runs.begin(), c->fe_runs.end() - kFrontEndEntries);
    return e;
}

// The run's moments into its slot (read back with its audio).
int32_t fe_moments(rv_chain* c, uint64_t first_sample, uint32_t count) {
    RunSlot& sl = S(c);
    const uint64_t floats = (uint64_t)((count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK) * RV_IQ_MOMENTS_PER_CHUNK;
    if (floats == 0) return RV_OK;
    const uint64_t cap = (uint64_t)((c->config.max_run_samples + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK) *
                         RV_IQ_MOMENTS_PER_CHUNK;
    if (sl.sums_dev.count < cap)
        if (int32_t st = sl.sums_dev.alloc(cap)) return st;
    if (int32_t st = sl.sums_host.reserve(cap)) return st;
    const rv_iq_moments_params mp{c->raw_mask, (uint32_t)(first_sample & c->raw_mask), count};
    int32_t st = c->config.mode == RV_CHAIN_PLAIN
                     ? launch_iq_moments(c->stream, mp, c->cf32_ring.ptr, sl.sums_dev.ptr)
                     : launch_iq_moments_raw(c->stream, c->config.format, mp, c->raw.ptr, sl.sums_dev.ptr);
    if (st) return st;
    c->stats.launches += 1;
    if ((st = cuda_status(cudaMemcpyAsync(sl.sums_host.ptr, sl.sums_dev.ptr, floats * sizeof(float),
                                          cudaMemcpyDeviceToHost, c->stream),
                          "front-end moments read-back")))
        return st;
    sl.sums_count = count;
    sl.sums_run = c->run_index;
    sl.sums_pending = true;
    return RV_OK;
}

// The table of corrections the fused kernel applies over a coarse window that
// starts at source sample `window` (which may precede the stream): the runs
// the window reaches, from the latest that began at or before its start.
// Uploaded into the run's slot; c->fe_table is null when none applies.
int32_t fe_table(rv_chain* c, int64_t window, bool keep_pointer) {
    c->fe_table = nullptr;
    auto& runs = c->fe_runs;
    // runs wholly before the window can no longer be read
    size_t drop = 0;
    while (drop + 1 < runs.size() && (int64_t)runs[drop + 1].start <= window) ++drop;
    runs.erase(runs.begin(), runs.begin() + (ptrdiff_t)drop);
    bool any = false;
    for (const auto& r : runs) any = any || r.entry.on;
    if (!any && !keep_pointer) return RV_OK;
    if (runs.size() > kFrontEndEntries)
        return set_error_fmt(RV_ERR_UNSUPPORTED,
                             "rv_chain_run: the channelizer's history spans %zu runs, more than the %u the front-end "
                             "correction keeps: use longer runs",
                             runs.size(), kFrontEndEntries);
    RunSlot& sl = S(c);
    if (sl.fe_dev.count == 0)
        if (int32_t st = sl.fe_dev.alloc(1)) return st;
    if (int32_t st = sl.fe_host.reserve(1)) return st;
    FrontEndTable* t = sl.fe_host.ptr;
    memset(t, 0, sizeof *t);
    t->count = runs.empty() ? 1u : (uint32_t)runs.size();
    if (runs.empty()) t->e[0] = FrontEndEntry{0u, 0u, 0.0F, 0.0F, 0.0F, 1.0F};
    for (size_t k = 0; k < runs.size(); ++k) {
        t->e[k] = runs[k].entry;
        const int64_t rel = (int64_t)runs[k].start - window;
        t->e[k].rel_start = rel > 0 ? (uint32_t)rel : 0u;
    }
    if (int32_t st = cuda_status(cudaMemcpyAsync(sl.fe_dev.ptr, t, sizeof *t, cudaMemcpyHostToDevice, c->stream),
                                 "front-end table upload"))
        return st;
    c->fe_table = sl.fe_dev.ptr;
    return RV_OK;
}

// Graph::plan_impulse_excision (core/engine/graph.cpp:1468-1488): the plan of
// this run's excision passes, or null while the stage is off. Switching it on
// restarts the cursor, which then waits for a full reference window.
const rv_excision_plan* plan_excision(rv_chain* c, uint64_t start, uint64_t count) {
    if (!c->ex_on) {
        c->ex_was_on = false;
        return nullptr;
    }
    if (!c->ex_was_on) c->ex_cursor.running = 0;
    c->ex_was_on = true;
    (void)rv_excision_plan_block(&c->ex_cursor, start, (uint32_t)count, &c->ex_plan);
    return &c->ex_plan;
}

// Graph::record_impulse_excision: the plan's passes, in place on `ring`.
int32_t excise(rv_chain* c, const rv_excision_plan& plan, rv_cf32* ring) {
    const uint64_t n = (uint64_t)c->raw_mask + 1u;
    if (int32_t st = rv_excise_block(c->stream, &c->ex_cfg, &plan, ring, n, c->ex_seg_power.ptr, c->ex_seg_level.ptr,
                                     c->ex_seg_power.count, c->ex_flags.ptr, c->ex_flags.count, c->ex_removed.ptr,
                                     c->ex_removed.count, c->ex_counters.ptr))
        return st;
    for (const rv_excision_params* q : {&plan.segment, &plan.reference, &plan.flag, &plan.apply})
        if (q->count) c->stats.launches += 1;
    c->ex_examined += plan.apply.count;
    return RV_OK;
}

// Graph::on_block's spectrum frame (core/engine/graph.cpp:5077-5095,
// 5218-5286): when the run completed N or more channel blocks, one frame of
// the last N (central half of each channel's N-point transform, dB), covering
// source samples [first * D - group delay, + N * D); then the attached
// detector consumes it on the device.
int32_t spectrum_frame(rv_chain* c, uint64_t first_block, uint32_t blocks) {
    if (c->spec_n == 0 || blocks == 0) return RV_OK;
    const uint64_t one_past = first_block + blocks, n = c->spec_n;
    if (one_past < n) return RV_OK;
    const uint64_t sfb = one_past - n;
    const rv_grid_params& g = c->config.grid;
    rv_spectrum_params sp{g.channels, c->spec_n, ilog2(c->spec_n), c->chan_blocks, c->chan_blocks - 1u,
                          (uint32_t)(sfb & (c->chan_blocks - 1u))};
    // the attached detector averages frames asynchronously on its own stream:
    // the previous frame must be read before this one overwrites it
    if (c->detector != nullptr)
        if (int32_t st = detector_release_to(c->detector, c->stream)) return st;
    if (int32_t st = rv_spectrum(c->stream, &sp, c->channel.ptr, c->channel.count, c->spec_twiddles.ptr,
                                 c->spec_twiddles.count, c->spec_window.ptr, c->spec_window.count, c->spec_frame.ptr,
                                 c->spec_frame.count))
        return st;
    c->stats.launches += 1;
    c->spec_start = sfb * g.decimation - c->group_delay;
    c->spec_count = n * g.decimation;
    c->spec_sequence += 1;
    c->spec_recorded = true;
    if (c->detector != nullptr) {
        if (int32_t st = detector_wait_for(c->detector, c->stream)) return st;
        uint32_t decisions = 0;
        if (int32_t st = rv_detector_consume_frames(c->detector, c->spec_frame.ptr, 1, c->spec_start, 0, c->spec_count,
                                                    1, &decisions))
            return st;
    }
    return RV_OK;
}

int32_t upload_table(rv_chain* c) {
    std::vector<RxDev> table(c->rx.size());
    for (size_t i = 0; i < c->rx.size(); ++i) {
        Receiver& r = c->rx[i];
        RxDev& d = table[i];
        memset(&d, 0, sizeof d);
        const rv_vrx_plan_info& p = r.plan;
        d.chan_base = p.placement.channel * c->chan_blocks;
        d.chan_mask = c->chan_blocks - 1u;
        d.taps = p.fine.taps;
        d.period = r.period;
        d.step_whole = (uint32_t)(p.channel_rate / p.demod_rate);
        d.step_rem = (uint32_t)(p.channel_rate % p.demod_rate);
        d.out_rate = (uint32_t)p.demod_rate;
        d.nco_log2 = p.fine.nco_log2;
        d.nco_delta = p.fine_nco_delta;
        d.lerped = r.d_lerped.ptr;
        d.taps_raw = reinterpret_cast<const float2*>(r.d_taps.ptr);
        d.phases = p.fine.phases;
        d.inv_out_rate = 1.0f / (float)p.demod_rate;
        d.nco = reinterpret_cast<const float2*>(c->nco.ptr);
        d.fine = reinterpret_cast<float2*>(r.d_fine.ptr);
        d.fine_mask = r.fine_mask;
        d.mode = p.demod.mode;
        d.decimation = p.demod.decimation;
        d.audio_taps = p.demod.audio_taps;
        d.dc_taps = p.demod.dc_taps;
        d.channels = p.demod.channels;
        d.pilot_taps = p.demod.pilot_taps;
        d.gain = p.demod_gain;
        d.reach = r.reach;
        d.weights = r.d_weights.ptr;
        d.det = r.d_det.ptr;
        d.carrier_state = r.d_state.ptr;
        d.carrier = p.carrier_loop;
        d.carrier_power = p.carrier.power;
        d.tile_cols = r.tile_cols;
        d.tile_block = r.tile_block;
        d.tile_rows = r.tile_rows;
        d.tile_buffers = r.tile_buffers;
        d.tile_seg = r.tile_seg;
        d.tile_stride = r.tile_stride;
        d.tile_period = r.tile_period;
        d.det_item = r.max_det_item;
        d.audio_item = r.max_audio_item;
        d.row_step = r.row_step;
        d.tc_chunks = r.tc_chunks;
        d.tc_b = r.d_tc.ptr;
    }
    if (c->rx_table.count < table.size())
        if (int32_t st = c->rx_table.alloc(table.size())) return st;
    if (!table.empty())
        if (int32_t st = cuda_status(cudaMemcpyAsync(c->rx_table.ptr, table.data(), table.size() * sizeof(RxDev),
                                                     cudaMemcpyHostToDevice, c->stream),
                                     "receiver table upload"))
            return st;
    c->table_dirty = false;
    return RV_OK;
}

// Copy `count` samples of native-format input into ring positions starting
// at `pos` (wrapping). `where` 0 = host memory, 1 = device memory.
int32_t copy_into_ring(rv_chain* c, uint8_t* ring, uint64_t ring_samples, uint64_t pos, const uint8_t* src,
                       uint64_t count, int32_t where) {
    const uint64_t bps = c->bytes_per_sample;
    const cudaMemcpyKind kind = where ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    // pipelined: on the copy stream, overlapping the previous run's kernels
    // (the ring holds two runs beyond the filter history, so this run's
    // samples never land where a run still in flight reads)
    cudaStream_t s = pipelined(c) ? c->copy_stream : c->stream;
    uint64_t done = 0;
    while (done < count) {
        const uint64_t at = (pos + done) % ring_samples;
        const uint64_t n = std::min<uint64_t>(count - done, ring_samples - at);
        if (int32_t st = cuda_status(cudaMemcpyAsync(ring + at * bps, src + done * bps, n * bps, kind, s), "input copy"))
            return st;
        done += n;
    }
    if (pipelined(c)) {
        if (int32_t st = cuda_status(cudaEventRecord(c->input_ready, s), "input event")) return st;
        if (int32_t st = cuda_status(cudaStreamWaitEvent(c->stream, c->input_ready, 0), "input wait")) return st;
    }
    return RV_OK;
}

int32_t coarse_plain(rv_chain* c, uint64_t first_sample, const uint8_t* src, uint64_t count, int32_t where,
                     uint64_t first_block, uint32_t blocks, const rv_excision_plan* excision) {
    const rv_grid_params& g = c->config.grid;
    // staging copy of this run's raw bytes, then convert into the cf32 ring
    if (int32_t st = copy_into_ring(c, c->raw.ptr, count + 1, 0, src, count, where)) return st;
    mark(c, 1);
    rv_convert_params cp{c->raw_mask, (uint32_t)first_sample, 0u, (uint32_t)count};
    if (int32_t st = rv_convert(c->stream, c->config.format, &cp, c->raw.ptr, c->raw.count, c->cf32_ring.ptr,
                                c->cf32_ring.count))
        return st;
    c->stats.launches += 1;
    // front end: moments of the converted run, then the run corrected in place
    bool fe_on = false;
    const FrontEndEntry fe = fe_prepare(c, first_sample, count, &fe_on);
    if (fe_on) {
        if (int32_t st = fe_moments(c, first_sample, (uint32_t)count)) return st;
        if (fe.on) {
            rv_iq_correct_params ip{c->raw_mask, (uint32_t)(first_sample & c->raw_mask), (uint32_t)count,
                                    fe.dc_i, fe.dc_q, fe.cross, fe.scale};
            if (int32_t st = rv_iq_correct(c->stream, &ip, c->cf32_ring.ptr, c->cf32_ring.count, c->cf32_ring.ptr,
                                           c->cf32_ring.count))
                return st;
            c->stats.launches += 1;
        }
    }
    // impulse excision in place on the corrected ring
    if (excision != nullptr)
        if (int32_t st = excise(c, *excision, c->cf32_ring.ptr)) return st;
    if (blocks == 0) return RV_OK;
    rv_pfb_branch_params bp{c->raw_mask, (uint32_t)(first_block * g.decimation), blocks};
    if (int32_t st = rv_pfb_branch(c->stream, &g, &bp, c->proto.ptr, c->proto.count, c->cf32_ring.ptr,
                                   c->cf32_ring.count, c->branch.ptr, c->branch.count))
        return st;
    rv_pfb_fft_params fp{g.channels, g.decimation, ilog2(g.channels), (uint32_t)first_block, blocks, c->chan_blocks,
                         c->chan_blocks - 1u};
    if (int32_t st = rv_pfb_fft(c->stream, &fp, c->branch.ptr, c->branch.count, c->twiddles.ptr, c->twiddles.count,
                                c->channel.ptr, c->channel.count))
        return st;
    c->stats.launches += 2;
    return RV_OK;
}

// With `deferred`, the coarse parameters are returned for a captured run to
// hand to its graph instead of being launched here.
int32_t coarse_batched(rv_chain* c, uint64_t first_sample, const uint8_t* src, uint64_t count, int32_t where,
                       uint64_t first_block, uint32_t blocks, rv_coarse_params* deferred,
                       const rv_excision_plan* excision) {
    const rv_grid_params& g = c->config.grid;
    if (int32_t st = copy_into_ring(c, c->raw.ptr, (uint64_t)c->raw_mask + 1u, first_sample, src, count, where))
        return st;
    mark(c, 1);
    // front end: moments of the run's raw samples (the fused kernel below
    // corrects every sample it converts with its run's parameters)
    bool fe_on = false;
    (void)fe_prepare(c, first_sample, count, &fe_on);
    if (fe_on)
        if (int32_t st = fe_moments(c, first_sample, (uint32_t)count)) return st;
    const int64_t window = (int64_t)(first_block * g.decimation) - (int64_t)((uint64_t)g.channels * g.taps_per_branch - 1u);
    const bool clean = c->ex_clean;
    if (clean) {
        // the run's samples into the cf32 ring, converted and corrected as the
        // fused kernel would, then excised in place; on a restart also the
        // channelizer's history behind them, which the ring does not hold yet
        uint64_t from = first_sample;
        if (c->ex_converted_end != first_sample) from = std::min<uint64_t>(from, window > 0 ? (uint64_t)window : 0u);
        const int64_t table_at = std::min<int64_t>((int64_t)from, window);
        if (int32_t st = fe_table(c, table_at, false)) return st;
        if (int32_t st = launch_convert_ring(c->stream, c->config.format, c->raw.ptr, c->raw_mask, (uint32_t)from,
                                             (uint32_t)(first_sample + count - from), (uint32_t)table_at, c->fe_table,
                                             c->clean.ptr))
            return st;
        c->stats.launches += 1;
        c->fe_table = nullptr;  // applied: the coarse kernel reads corrected samples
        c->ex_converted_end = first_sample + count;
        if (excision != nullptr)
            if (int32_t st = excise(c, *excision, c->clean.ptr)) return st;
    }
    if (blocks == 0) return RV_OK;
    // a captured graph reads the table whenever front-end correction is on
    if (!clean)
        if (int32_t st = fe_table(c, window, c->graph && fe_on)) return st;
    // stream-start history reads as zero, as the plain path's zeroed ring does
    const uint64_t support = (uint64_t)g.channels * g.taps_per_branch - 1u;
    const uint64_t centre = first_block * g.decimation;
    const uint32_t lead_zero = centre >= support ? 0u : (uint32_t)(support - centre);
    rv_coarse_params p{c->raw_mask, (uint32_t)(first_block * g.decimation) & c->raw_mask, blocks, (uint32_t)first_block,
                       c->chan_blocks, c->chan_blocks - 1u, lead_zero};
    if (deferred != nullptr) {
        *deferred = p;
        return RV_OK;
    }
    if (!c->fused) {
        // no fused kernel for this grid: the reference's two dispatches over
        // the clean ring (stream-start history is the ring's zeroed slots)
        rv_pfb_branch_params bp{c->raw_mask, (uint32_t)(first_block * g.decimation), blocks};
        if (int32_t st = rv_pfb_branch(c->stream, &g, &bp, c->proto.ptr, c->proto.count, c->clean.ptr, c->clean.count,
                                       c->branch.ptr, c->branch.count))
            return st;
        rv_pfb_fft_params fp{g.channels, g.decimation, ilog2(g.channels), (uint32_t)first_block, blocks,
                             c->chan_blocks, c->chan_blocks - 1u};
        if (int32_t st = rv_pfb_fft(c->stream, &fp, c->branch.ptr, c->branch.count, c->twiddles.ptr, c->twiddles.count,
                                    c->channel.ptr, c->channel.count))
            return st;
        c->stats.launches += 2;
        return RV_OK;
    }
    if (int32_t st = launch_coarse_fused(c->stream, g, clean ? kFormatCf32Ring : c->config.format, p,
                                         clean ? static_cast<const void*>(c->clean.ptr) : c->raw.ptr, c->proto.ptr,
                                         c->twiddles.ptr, c->channel.ptr, nullptr, c->fe_table))
        return st;
    c->stats.launches += 1;
    return RV_OK;
}

// The 2D tile shape of a receiver's fine stage (fine_tiles.cu): rows of P'
// outputs (the pattern period times the smallest k making it 48 or more), cut
// into column blocks of at most 16 R columns (16 slots of R adjacent columns),
// chunks of 16 rows, one or two chunks staged, the block's table slice and
// row segments in shared memory. A shape changes which thread computes which
// output and what is staged, never an output's arithmetic.
struct TileShape {
    uint32_t cols = 0, block = 0, rows = 0, buffers = 0, seg = 0, stride = 0, period = 0, shared = 0;
    uint64_t row_step = 0;
    double score = 0.0;  // the rule's preference: column slots filled, then larger R, then two buffers
    bool same(const TileShape& o) const {
        return cols == o.cols && block == o.block && rows == o.rows && buffers == o.buffers && seg == o.seg &&
               stride == o.stride && period == o.period && shared == o.shared;
    }
};

// Every tile shape of a receiver that fits `budget` float2 of shared memory,
// R = 4..1, two staged chunks before one.
void tile_shapes(const Receiver& r, uint64_t fc, uint64_t fd, uint32_t budget, std::vector<TileShape>& out) {
    const uint64_t T = r.plan.fine.taps;
    if (r.period == 0) return;
    const uint64_t P = (uint64_t)r.period * ((48u + r.period - 1u) / r.period);
    if (P > 65535u || (P * fc) % fd != 0) return;
    for (uint32_t R = 4; R >= 1; --R) {
        const uint64_t cap = (uint64_t)kTileSlots * R;
        const uint64_t nblk = (P + cap - 1u) / cap;
        const uint64_t A = (P + nblk - 1u) / nblk;
        uint64_t L = 0;
        for (uint64_t a0 = 0; a0 < P; a0 += A) {
            const uint64_t w = std::min<uint64_t>(A, P - a0);
            L = std::max<uint64_t>(L, (a0 + w - 1u) * fc / fd - a0 * fc / fd + T);
        }
        const uint64_t Lp = L | 1u;
        // every block runs all 16 slots of R columns
        const double fill = (double)P / (double)(nblk * kTileSlots * R);
        for (uint32_t nb = 2; nb >= 1; --nb) {
            const uint64_t need = (T + 1u) / 2u * 2u * A + (uint64_t)nb * kTileRows * Lp;  // tap pairs + rows
            if (need > budget) continue;
            TileShape sh;
            sh.cols = (uint32_t)A;
            sh.block = (uint32_t)A;
            sh.rows = R;
            sh.buffers = nb;
            sh.seg = (uint32_t)L;
            sh.stride = (uint32_t)Lp;
            sh.period = (uint32_t)P;
            sh.shared = (uint32_t)need;
            sh.row_step = P * fc / fd;
            sh.score = fill * (1.0 + 0.01 * R) * (nb == 2 ? 1.0 : 0.97);
            out.push_back(sh);
        }
    }
}

void set_tile_shape(Receiver& r, const TileShape& sh) {
    r.tile_cols = sh.cols;
    r.tile_block = sh.block;
    r.tile_rows = sh.rows;
    r.tile_buffers = sh.buffers;
    r.tile_seg = sh.seg;
    r.tile_stride = sh.stride;
    r.row_step = sh.row_step;
    r.tile_period = sh.period;
    r.tile_shared = sh.shared;
}

// The rule's shape: among those that fit `budget`, the one that leaves the
// fewest column slots idle (then the larger R, then two buffers). Leaves
// tile_cols at 0 (not tiled) when nothing fits. rv_chain_autotune replaces
// the rule's choice by timing.
void plan_tiles(Receiver& r, uint64_t fc, uint64_t fd, uint32_t budget) {
    r.tile_cols = 0;
    std::vector<TileShape> shapes;
    tile_shapes(r, fc, fd, budget, shapes);
    const TileShape* best = nullptr;
    for (const TileShape& sh : shapes)
        if (best == nullptr || sh.score > best->score) best = &sh;
    if (best != nullptr) set_tile_shape(r, *best);
}

// Tiles covering fine outputs [first, first + count) of receiver `rx`: every
// column block over the rows those outputs touch, rows split so a tile costs
// about `target` complex MACs (at least two row chunks).
void push_tiles(std::vector<FineTile>& list, uint32_t rx, const Receiver& r, uint64_t first, uint64_t count,
                uint64_t target) {
    if (count == 0) return;
    if (r.tc_chunks != 0) {
        // fast mode: GEMM tiles of kFineTcRows rows by kFineTcColumns columns
        const uint64_t P = r.tile_period, end = first + count;
        const uint64_t row_lo = first / P, row_hi = (end - 1u) / P + 1u;
        for (uint64_t b = row_lo; b < row_hi; b += kFineTcRows)
            for (uint64_t a0 = 0; a0 < P; a0 += kFineTcColumns) {
                FineTile t{};
                t.rx = rx;
                t.a0 = (uint32_t)a0;
                t.width = (uint32_t)std::min<uint64_t>(kFineTcColumns, P - a0);
                t.rows = (uint32_t)std::min<uint64_t>(kFineTcRows, row_hi - b);
                t.row0 = b;
                t.first = first;
                t.end = end;
                list.push_back(t);
            }
        return;
    }
    const uint64_t P = r.tile_period, T = r.plan.fine.taps, end = first + count;
    const uint64_t row_lo = first / P, row_hi = (end - 1u) / P + 1u;
    const uint64_t chunk = kTileRows;
    for (uint64_t a0 = 0; a0 < P; a0 += r.tile_block) {
        const uint64_t w = std::min<uint64_t>(r.tile_block, P - a0);
        uint64_t rows = std::max<uint64_t>(2u * chunk, target / std::max<uint64_t>(1u, w * T));
        rows = (rows + chunk - 1u) / chunk * chunk;
        for (uint64_t b = row_lo; b < row_hi; b += rows) {
            FineTile t{};
            t.rx = rx;
            t.a0 = (uint32_t)a0;
            t.width = (uint32_t)w;
            t.rows = (uint32_t)std::min<uint64_t>(rows, row_hi - b);
            t.row0 = b;
            t.first = first;
            t.end = end;
            list.push_back(t);
        }
    }
}

// Fine items carry the exact input index of their first output and its
// resampler fraction (resample_block, core/dsp/vrx_reference.cpp:2786-2810)
// so the device does no 64-bit division. Returns the largest window.
uint32_t push_fine_items(std::vector<WorkItem>& list, uint32_t rx, const Receiver& r, uint64_t first, uint64_t count,
                         uint32_t per_item) {
    const uint64_t fc = (uint64_t)r.plan.channel_rate, fd = (uint64_t)r.plan.demod_rate;
    const uint64_t step_whole = fc / fd, step_rem = fc % fd;
    auto input_of = [&](uint64_t j, uint64_t* frac) {
        const uint64_t whole = j / fd, part = j % fd, cp = part * step_rem;
        if (frac) *frac = cp % fd;
        return j * step_whole + whole * step_rem + cp / fd;
    };
    uint32_t widest = 0;
    uint64_t done = 0;
    while (done < count) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(count - done, per_item);
        WorkItem w{};
        w.rx = rx;
        w.count = n;
        w.first = first + done;
        uint64_t frac0 = 0;
        w.n0 = input_of(w.first, &frac0);
        w.frac0 = (uint32_t)frac0;
        w.p0 = (uint32_t)(w.first % r.period);
        const uint64_t n_last = input_of(w.first + n - 1u, nullptr);
        w.window = (uint32_t)(n_last - w.n0) + r.plan.fine.taps;
        widest = std::max(widest, w.window);
        list.push_back(w);
        done += n;
    }
    return widest;
}

// Section offsets of the work lists in the device item array of a captured
// run: fine, carrier, detector, audio, then the unit items.
struct Sections {
    size_t fine, carrier, unit, total;
    explicit Sections(const GraphShape& sh)
        : fine(0), carrier(sh.fine), unit(carrier + sh.carrier), total(unit + sh.unit_items) {}
};

// This run's detector and audio spans per receiver (the batched detector and
// audio kernels cut them into items on the device).
struct SpanTable {
    std::vector<RxRun> runs;
    std::vector<uint32_t> det_prefix, audio_prefix;
    uint32_t det_total = 0, audio_total = 0;
};

size_t span_bytes(size_t nrx) { return nrx * sizeof(RxRun) + 2u * (nrx + 1u) * sizeof(uint32_t); }

// Device addresses of the span table's parts for `nrx` receivers.
void span_lists(rv_chain* c, uint32_t nrx, SpanList* det, SpanList* audio) {
    const uint8_t* base = S(c).spans_dev.ptr;
    const RxRun* runs = reinterpret_cast<const RxRun*>(base);
    const uint32_t* dp = reinterpret_cast<const uint32_t*>(base + nrx * sizeof(RxRun));
    *det = SpanList{runs, dp, nrx, 0u};
    *audio = SpanList{runs, dp + nrx + 1u, nrx, 1u};
}

// Copies the span table to the device (capacity kept from earlier runs).
int32_t upload_spans(rv_chain* c, const SpanTable& t) {
    const size_t nrx = t.runs.size(), bytes = span_bytes(nrx);
    if (S(c).spans_dev.count < bytes)
        if (int32_t st = S(c).spans_dev.alloc(bytes + bytes / 2)) return st;
    if (int32_t st = S(c).spans_host.reserve(bytes + bytes / 2)) return st;
    uint8_t* h = S(c).spans_host.ptr;
    memcpy(h, t.runs.data(), nrx * sizeof(RxRun));
    memcpy(h + nrx * sizeof(RxRun), t.det_prefix.data(), (nrx + 1u) * sizeof(uint32_t));
    memcpy(h + nrx * sizeof(RxRun) + (nrx + 1u) * sizeof(uint32_t), t.audio_prefix.data(), (nrx + 1u) * sizeof(uint32_t));
    return cuda_status(cudaMemcpyAsync(S(c).spans_dev.ptr, h, bytes, cudaMemcpyHostToDevice, c->stream), "span upload");
}

// Records the coarse kernel and every batched receiver kernel, reading their
// counts and the coarse parameters from S(c).counts_dev, into one graph.
int32_t capture(rv_chain* c, const rv_coarse_params& coarse) {
    const GraphShape& sh = S(c).shape;
    const Sections o(sh);
    RunCounts* rc = S(c).counts_dev.ptr;
    const float2* chan = reinterpret_cast<const float2*>(c->channel.ptr);
    WorkItem* items = S(c).items_dev.ptr;
    cudaGraph_t graph = nullptr;
    if (int32_t st = cuda_status(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed), "graph capture begin"))
        return st;
    int32_t st = launch_coarse_fused(c->stream, c->config.grid, sh.excision ? kFormatCf32Ring : c->config.format, coarse,
                                     sh.excision ? static_cast<const void*>(c->clean.ptr) : c->raw.ptr, c->proto.ptr,
                                     c->twiddles.ptr, c->channel.ptr, &rc->coarse,
                                     sh.front_end ? S(c).fe_dev.ptr : nullptr);
    if (!st)
        st = c->fast ? launch_fine_tc(c->stream, c->rx_table.ptr, S(c).tiles_dev.ptr, sh.tiles, chan, &rc->queues.tiles,
                                      &rc->tiles, c->tc_status.ptr)
                     : launch_fine_tiles(c->stream, c->rx_table.ptr, S(c).tiles_dev.ptr, sh.tiles, chan, sh.tile_shared,
                                         &rc->queues.tiles, &rc->tiles);
    if (!st)
        st = launch_fine_units(c->stream, c->rx_table.ptr, items, S(c).units_dev.ptr, sh.units, chan, c->unit_budget,
                               &rc->queues.units, &rc->units);
    if (!st)
        st = launch_fine_batched(c->stream, c->rx_table.ptr, items + o.fine, sh.fine, chan, sh.fine_window,
                                 &rc->queues.fine, &rc->fine);
    if (!st) st = launch_carrier_batched(c->stream, c->rx_table.ptr, items + o.carrier, sh.carrier, &rc->carrier);
    SpanList det, audio;
    span_lists(c, sh.nrx, &det, &audio);
    if (!st)
        st = launch_detect_batched(c->stream, c->rx_table.ptr, det, sh.nrx, kDetWindow, &rc->queues.detect,
                                   &rc->detect, c->fast);
    if (!st)
        st = launch_audio_batched(c->stream, c->rx_table.ptr, audio, sh.nrx, S(c).audio_dev.ptr, kDetWindow,
                                  sh.weights_cap, &rc->queues.audio, &rc->audio, c->fast);
    const int32_t end = cuda_status(cudaStreamEndCapture(c->stream, &graph), "graph capture end");
    if (st || end) {
        if (graph) cudaGraphDestroy(graph);
        return st ? st : end;
    }
    st = cuda_status(cudaGraphInstantiate(&S(c).exec, graph, 0), "graph instantiate");
    cudaGraphDestroy(graph);
    if (st) {
        S(c).exec = nullptr;
        return st;
    }
    c->stats.graph_captures += 1;
    return RV_OK;
}

// A captured run: upload this run's counts and work lists into the sections
// the graph reads, capture first when the graph is missing or too small, then
// replay it with one launch.
int32_t run_captured(rv_chain* c, const rv_coarse_params& coarse, const std::vector<WorkItem>& fine,
                     const std::vector<WorkItem>& carrier, const SpanTable& spans,
                     const std::vector<WorkItem>& unit_items, const std::vector<FineUnit>& units,
                     const std::vector<FineTile>& tiles, uint32_t fine_window) {
    const uint32_t window = std::min<uint32_t>(kFineWindow, (fine_window + 255u) & ~255u);
    GraphShape& sh = S(c).shape;
    const uint32_t nrx = (uint32_t)spans.runs.size();
    if (int32_t st = upload_spans(c, spans)) return st;
    const bool fits = S(c).exec != nullptr && fine.size() <= sh.fine && carrier.size() <= sh.carrier &&
                      sh.nrx == nrx && sh.spans_ptr == S(c).spans_dev.ptr && unit_items.size() <= sh.unit_items &&
                      sh.front_end == (c->fe_table != nullptr ? 1u : 0u) && sh.excision == (c->ex_clean ? 1u : 0u) &&
                      units.size() <= sh.units && tiles.size() <= sh.tiles && sh.tile_shared == c->tile_shared &&
                      sh.tiles_ptr == S(c).tiles_dev.ptr && window <= sh.fine_window && sh.weights_cap == c->weights_cap &&
                      sh.unit_budget == c->unit_budget && sh.audio_ptr == S(c).audio_dev.ptr &&
                      sh.table_ptr == c->rx_table.ptr && sh.items_ptr == S(c).items_dev.ptr &&
                      sh.units_ptr == S(c).units_dev.ptr;
    if (!fits) {
        if (S(c).exec) cudaGraphExecDestroy(S(c).exec);
        S(c).exec = nullptr;
        auto grow = [](size_t need, uint32_t old) {
            return (uint32_t)std::max<size_t>(old, need == 0 ? 0 : need + need / 2 + 16);
        };
        GraphShape n;
        n.fine = grow(fine.size(), sh.fine);
        n.carrier = grow(carrier.size(), sh.carrier);
        n.nrx = nrx;
        n.spans_ptr = S(c).spans_dev.ptr;
        n.front_end = c->fe_table != nullptr ? 1u : 0u;
        n.excision = c->ex_clean ? 1u : 0u;
        n.unit_items = grow(unit_items.size(), sh.unit_items);
        n.units = grow(units.size(), sh.units);
        n.tiles = grow(tiles.size(), sh.tiles);
        n.tile_shared = c->tile_shared;
        n.fine_window = std::max(window, sh.fine_window);
        n.weights_cap = c->weights_cap;
        n.unit_budget = c->unit_budget;
        const size_t total = Sections(n).total;
        if (S(c).items_dev.count < total + 1)
            if (int32_t st = S(c).items_dev.alloc(total + 1)) return st;
        if (S(c).units_dev.count < (size_t)n.units + 1)
            if (int32_t st = S(c).units_dev.alloc(n.units + 1)) return st;
        if (S(c).tiles_dev.count < (size_t)n.tiles + 1)
            if (int32_t st = S(c).tiles_dev.alloc(n.tiles + 1)) return st;
        if (S(c).counts_dev.count == 0)
            if (int32_t st = S(c).counts_dev.alloc(1)) return st;
        n.audio_ptr = S(c).audio_dev.ptr;
        n.table_ptr = c->rx_table.ptr;
        n.items_ptr = S(c).items_dev.ptr;
        n.units_ptr = S(c).units_dev.ptr;
        n.tiles_ptr = S(c).tiles_dev.ptr;
        sh = n;
    }
    const Sections o(sh);
    if (int32_t st = S(c).items_host.reserve(o.total + 1)) return st;
    if (int32_t st = S(c).units_host.reserve((size_t)sh.units + 1)) return st;
    if (int32_t st = S(c).tiles_host.reserve((size_t)sh.tiles + 1)) return st;
    if (int32_t st = S(c).counts_host.reserve(1)) return st;
    RunCounts* rc = S(c).counts_host.ptr;
    memset(rc, 0, sizeof *rc);
    rc->units = (uint32_t)units.size();
    rc->fine = (uint32_t)fine.size();
    rc->carrier = (uint32_t)carrier.size();
    rc->detect = spans.det_total;
    rc->audio = spans.audio_total;
    rc->tiles = (uint32_t)tiles.size();
    rc->coarse = coarse;
    if (int32_t st = cuda_status(cudaMemcpyAsync(S(c).counts_dev.ptr, rc, sizeof *rc, cudaMemcpyHostToDevice, c->stream),
                                 "run counts upload"))
        return st;
    const std::pair<const std::vector<WorkItem>*, size_t> lists[] = {
        {&fine, o.fine}, {&carrier, o.carrier}, {&unit_items, o.unit}};
    for (const auto& l : lists) {
        if (l.first->empty()) continue;
        WorkItem* h = S(c).items_host.ptr + l.second;
        memcpy(h, l.first->data(), l.first->size() * sizeof(WorkItem));
        if (int32_t st = cuda_status(cudaMemcpyAsync(S(c).items_dev.ptr + l.second, h, l.first->size() * sizeof(WorkItem),
                                                     cudaMemcpyHostToDevice, c->stream),
                                     "work list upload"))
            return st;
    }
    if (!units.empty()) {
        for (size_t i = 0; i < units.size(); ++i) {
            S(c).units_host.ptr[i] = units[i];
            S(c).units_host.ptr[i].first_item += (uint32_t)o.unit;
        }
        if (int32_t st = cuda_status(cudaMemcpyAsync(S(c).units_dev.ptr, S(c).units_host.ptr, units.size() * sizeof(FineUnit),
                                                     cudaMemcpyHostToDevice, c->stream),
                                     "unit upload"))
            return st;
    }
    if (!tiles.empty()) {
        memcpy(S(c).tiles_host.ptr, tiles.data(), tiles.size() * sizeof(FineTile));
        if (int32_t st = cuda_status(cudaMemcpyAsync(S(c).tiles_dev.ptr, S(c).tiles_host.ptr, tiles.size() * sizeof(FineTile),
                                                     cudaMemcpyHostToDevice, c->stream),
                                     "tile upload"))
            return st;
    }
    if (S(c).exec == nullptr)
        if (int32_t st = capture(c, coarse)) return st;
    mark(c, 2);
    mark(c, 3);
    if (int32_t st = cuda_status(cudaGraphLaunch(S(c).exec, c->stream), "graph launch")) return st;
    mark(c, 4);
    c->stats.graph_launches += 1;
    c->stats.launches += 1 + (sh.units ? 1 : 0) + (sh.fine ? 1 : 0) + (sh.carrier ? 1 : 0) + (sh.nrx ? 2 : 0) +
                         (sh.tiles ? 1 : 0);
    c->stats.work_items += fine.size() + carrier.size() + spans.det_total + spans.audio_total + unit_items.size() +
                           tiles.size();
    return RV_OK;
}

}  // namespace

extern "C" {

int32_t rv_chain_create(rv_context* context, const rv_chain_config* config, rv_chain** out) {
    if (context == nullptr || config == nullptr || out == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: NULL argument");
    *out = nullptr;
    if (int32_t st = validate_grid(&config->grid)) return st;
    const rv_grid_params& g = config->grid;
    if (config->format != RV_FORMAT_CS16 && config->format != RV_FORMAT_CU8)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_chain_create: input format %d (cs16 and cu8 are supported)",
                             config->format);
    if (config->mode != RV_CHAIN_BATCHED && config->mode != RV_CHAIN_PLAIN && config->mode != RV_CHAIN_FAST &&
        config->mode != RV_CHAIN_HOISTED)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: mode %d", config->mode);
    if (config->mode == RV_CHAIN_HOISTED && config->pipelined)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: a hoisted chain runs its launches directly (pipelined = 0)");
    rv_chain_config cfg = *config;
    const bool fast = cfg.mode == RV_CHAIN_FAST, hoisted = cfg.mode == RV_CHAIN_HOISTED;
    if (fast || hoisted) cfg.mode = RV_CHAIN_BATCHED;  // the batched chain's state and bookkeeping
    config = &cfg;
    if (config->rate <= 0 || config->rate % g.decimation != 0)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: rate %lld must be a positive multiple of D=%u",
                             (long long)config->rate, g.decimation);
    if (config->max_run_samples == 0 || config->max_run_samples > (1u << 30))
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: max_run_samples must be in [1, 2^30]");
    if (config->pipelined > 1u || (config->pipelined && config->mode != RV_CHAIN_BATCHED))
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: pipelined runs are a batched-chain mode (pipelined = 1)");
    rv_chain* c = new (std::nothrow) rv_chain;
    if (c == nullptr) return set_error_fmt(RV_ERR_NO_MEMORY, "rv_chain_create: out of host memory");
    c->context = context;
    c->stream = reinterpret_cast<cudaStream_t>(rv_context_stream(context));
    c->config = *config;
    c->fast = fast;
    c->hoisted = hoisted;
    if (c->config.attenuation_db <= 0.0) c->config.attenuation_db = 120.0;
    rv_front_end_init(&c->fe);
    c->bytes_per_sample = config->format == RV_FORMAT_CS16 ? 4u : 2u;
    // the filter history, and room for the impulse excision's lag (the
    // channelizer then reads up to max_width + lead or a segment behind the
    // newest sample)
    const uint64_t history = (uint64_t)g.channels * g.taps_per_branch + g.decimation +
                             (uint64_t)RV_EXCISE_MAX_WIDTH + RV_EXCISE_MAX_GUARD + (1u << RV_EXCISE_MAX_SEG_LOG2);
    // pipelined: two runs in the ring beyond the history, so that a run's input
    // copy never overwrites samples the run before it still reads
    const uint64_t runs_held = config->pipelined ? 2u : 1u;
    const uint64_t raw_cap = bit_ceil64(runs_held * config->max_run_samples + history + 1u);
    if (raw_cap > (1ull << 31)) {
        delete c;
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_create: ring of %llu samples is too large", (unsigned long long)raw_cap);
    }
    c->raw_mask = (uint32_t)(raw_cap - 1u);
    const uint64_t blocks_per_run = config->max_run_samples / g.decimation + 2u;
    c->chan_blocks = (uint32_t)bit_ceil64(blocks_per_run + 256u + 8u);
    int32_t st = RV_OK;
    if (config->mode == RV_CHAIN_BATCHED) {
        st = c->raw.alloc(raw_cap * c->bytes_per_sample);
        if (!st) st = cuda_status(cudaMemsetAsync(c->raw.ptr, 0, raw_cap * c->bytes_per_sample, c->stream), "ring clear");
        c->fused = coarse_fused_supported(g);
        if (!st && !c->fused) {
            // the stream-start history reads as zero, as in the plain chain's ring
            st = c->clean.alloc(raw_cap);
            if (!st) st = cuda_status(cudaMemsetAsync(c->clean.ptr, 0, raw_cap * sizeof(rv_cf32), c->stream), "ring clear");
            if (!st) st = c->branch.alloc(blocks_per_run * g.channels);
            c->ex_clean = true;
            c->ex_converted_end = ~0ull;
        }
    } else {
        st = c->raw.alloc(((uint64_t)config->max_run_samples + 1u) * c->bytes_per_sample);
        if (!st) st = c->cf32_ring.alloc(raw_cap);
        if (!st) st = cuda_status(cudaMemsetAsync(c->cf32_ring.ptr, 0, raw_cap * sizeof(rv_cf32), c->stream), "ring clear");
        if (!st) st = c->branch.alloc(blocks_per_run * g.channels);
    }
    if (!st) st = c->channel.alloc((uint64_t)g.channels * c->chan_blocks);
    if (!st && fast) st = c->tc_status.alloc(1);
    if (!st && fast) st = cuda_status(cudaMemsetAsync(c->tc_status.ptr, 0, sizeof(uint32_t), c->stream), "status clear");
    if (!st) st = cuda_status(cudaMemsetAsync(c->channel.ptr, 0, (uint64_t)g.channels * c->chan_blocks * sizeof(rv_cf32), c->stream),
                              "channel clear");
    std::vector<rv_cf32> tw, nco;
    if (!st) st = design_prototype_table(g, c->config.attenuation_db, c->proto_host);
    // the linear-phase prototype's delay: its design length (M (T - 1) + 1) over two
    c->group_delay = (uint64_t)g.channels * (g.taps_per_branch - 1u) / 2u;
    if (!st) st = build_twiddle_table(g.channels, tw);
    if (!st) st = build_nco(16, nco);
    if (!st) st = c->proto.alloc(c->proto_host.size());
    if (!st) st = c->twiddles.alloc(tw.size());
    if (!st) st = c->nco.alloc(nco.size());
    if (!st) st = cuda_status(cudaMemcpyAsync(c->proto.ptr, c->proto_host.data(), c->proto_host.size() * 4, cudaMemcpyHostToDevice, c->stream), "prototype upload");
    if (!st) st = cuda_status(cudaMemcpyAsync(c->twiddles.ptr, tw.data(), tw.size() * 8, cudaMemcpyHostToDevice, c->stream), "twiddle upload");
    if (!st) st = cuda_status(cudaMemcpyAsync(c->nco.ptr, nco.data(), nco.size() * 8, cudaMemcpyHostToDevice, c->stream), "nco upload");
    if (!st && c->config.profile)
        for (int i = 0; i < 6 && !st; ++i) st = cuda_status(cudaEventCreate(&c->marks[i]), "chain events");
    for (RunSlot& sl : c->slots)
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming), "chain events");
    if (!st && c->config.pipelined) {
        st = cuda_status(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "copy stream");
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&c->input_ready, cudaEventDisableTiming), "chain events");
    }
    if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "chain create");
    if (st) {
        rv_chain_destroy(c);
        return st;
    }
    *out = c;
    return clear_error();
}

int32_t rv_chain_destroy(rv_chain* c) {
    if (c == nullptr) return RV_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (Receiver& r : c->rx) {
        r.d_taps.release();
        r.d_lerped.release();
        r.d_tc.release();
        r.d_fine.release();
        r.d_det.release();
        r.d_weights.release();
        r.d_state.release();
    }
    c->raw.release();
    c->cf32_ring.release();
    c->clean.release();
    c->ex_seg_power.release();
    c->ex_seg_level.release();
    c->ex_flags.release();
    c->ex_counters.release();
    c->ex_removed.release();
    c->branch.release();
    c->channel.release();
    c->tc_status.release();
    c->hoisted_prefix.release();
    c->proto.release();
    c->twiddles.release();
    c->nco.release();
    c->rx_table.release();
    for (RunSlot& sl : c->slots) sl.release();
    c->spec_window.release();
    c->spec_twiddles.release();
    c->spec_frame.release();
    if (c->input_ready) cudaEventDestroy(c->input_ready);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (cudaEvent_t e : c->marks)
        if (e) cudaEventDestroy(e);
    delete c;
    return clear_error();
}

int32_t rv_chain_add_receiver(rv_chain* c, const rv_vrx_request* request, uint32_t* id) {
    if (c == nullptr || request == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_add_receiver: NULL");
    Receiver r;
    r.request = *request;
    if (int32_t st = plan_receiver(c->config.grid, c->config.rate, *request, r.plan, r.taps, r.weights)) return st;
    const rv_vrx_plan_info& p = r.plan;
    const uint64_t fc = (uint64_t)p.channel_rate, fd = (uint64_t)p.demod_rate;
    const uint64_t rem = fc % fd;
    r.period = (uint32_t)(fd / std::gcd(rem == 0 ? fd : rem, fd));
    r.fine_history = demod_fine_history(&p.demod);
    r.det_history = (p.demod.mode == RV_DEMOD_AM || p.demod.mode == RV_DEMOD_SAM) ? p.demod.dc_taps - 1u
                    : (p.demod.mode == RV_DEMOD_NFM || p.demod.mode == RV_DEMOD_WFM)   ? 1u
                                                                                        : 0u;
    r.reach = r.fine_history - r.det_history;
    // fine outputs one run can produce, plus history, plus a carry of one run
    const uint64_t blocks = c->config.max_run_samples / c->config.grid.decimation + 2u;
    const uint64_t max_fine = blocks * fd / fc + 2u;
    const uint64_t cap = bit_ceil64(2u * max_fine + r.fine_history + 1024u);
    if (cap > (1ull << 31)) return set_error_fmt(RV_ERR_INVALID, "rv_chain_add_receiver: fine ring too large");
    r.fine_mask = (uint32_t)(cap - 1u);
    // item sizes that keep every staged window inside shared memory
    const uint64_t step_max = fc / fd + 1u;
    r.max_fine_item = (uint32_t)std::min<uint64_t>(kMaxItem, (kFineWindow - p.fine.taps) / step_max + 1u);
    // AM / SAM run four DC-removal outputs per thread (window count + dc + 2)
    // (the other detectors also take four outputs per thread: bigger items,
    // fewer per-item queue and barrier steps)
    if (p.demod.mode == RV_DEMOD_AM || p.demod.mode == RV_DEMOD_SAM)
        r.max_det_item = (uint32_t)std::min<uint64_t>(4u * kMaxItem, kDetWindow - p.demod.dc_taps - 2u - 8u);
    else
        r.max_det_item = 4u * kMaxItem;
    const uint64_t dec = p.demod.decimation;
    if (r.reach + 1u > kDetWindow)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_chain_add_receiver: audio history %u exceeds the %u-sample window",
                             r.reach, kDetWindow);
    r.max_audio_item = (uint32_t)std::min<uint64_t>(kMaxItem, (kDetWindow - r.reach - 1u) / dec + 1u);
    int32_t st = r.d_taps.alloc(r.taps.size());
    if (!st) st = cuda_status(cudaMemcpyAsync(r.d_taps.ptr, r.taps.data(), r.taps.size() * 8, cudaMemcpyHostToDevice, c->stream), "taps upload");
    if (!st && c->config.mode == RV_CHAIN_BATCHED && (uint64_t)r.period * p.fine.taps <= kMaxLerpEntries) {
        st = r.d_lerped.alloc((uint64_t)r.period * p.fine.taps);
        if (!st)
            st = launch_lerp_table(c->stream, r.d_taps.ptr, r.d_lerped.ptr, p.fine.taps, p.fine.phases, r.period,
                                   (uint32_t)rem, (uint32_t)fd, 1.0f / (float)fd);
    }
    if (!st && r.d_lerped.ptr) {
        // the unit kernel keeps the whole blended table in shared memory when
        // it leaves room for a window of 256 outputs; otherwise half of shared
        // memory holds the window and the other half row chunks of the table
        if (c->unit_budget == 0) c->unit_budget = fine_unit_shared_budget();
        const uint64_t T = p.fine.taps;
        const uint64_t table = (uint64_t)r.period * T;
        const uint64_t min_window = 256u * step_max + T;
        uint64_t avail;
        if (table + min_window <= c->unit_budget) {
            r.table_rows = (uint32_t)T;
            avail = c->unit_budget - table;
        } else {
            avail = c->unit_budget / 2;
            r.table_rows = (uint32_t)std::min<uint64_t>(T, (c->unit_budget - avail) / r.period);
        }
        if (r.table_rows == 0 || avail < T + step_max) {
            r.max_unit_item = 0;  // the per-item kernel with taps from L2
        } else {
            r.max_unit_item = (uint32_t)std::min<uint64_t>(kUnitThreads, (avail - T) / step_max + 1u);
        }
        // the 2D tiles take over where a table slice and a chunk of rows fit;
        // a shape within `tile_share` of shared memory leaves room for more
        // CTAs per SM (measured: two per SM beat one with twice the rows)
        plan_tiles(r, fc, fd, c->unit_budget / kTileShare - 128u);
        if (r.tile_cols == 0) plan_tiles(r, fc, fd, c->unit_budget);
        if (r.tile_cols != 0) c->tile_shared = std::max(c->tile_shared, r.tile_shared);
    }
    if (!st) st = r.d_fine.alloc(cap);
    if (!st) st = cuda_status(cudaMemsetAsync(r.d_fine.ptr, 0, cap * sizeof(rv_cf32), c->stream), "fine clear");
    if (!st) st = r.d_det.alloc(cap);
    if (!st) st = cuda_status(cudaMemsetAsync(r.d_det.ptr, 0, cap * sizeof(float), c->stream), "det clear");
    if (!st) st = r.d_weights.alloc(r.weights.size());
    if (!st) st = cuda_status(cudaMemcpyAsync(r.d_weights.ptr, r.weights.data(), r.weights.size() * 4, cudaMemcpyHostToDevice, c->stream), "weights upload");
    if (!st) st = r.d_state.alloc(RV_CARRIER_STATE_WORDS);
    if (!st) st = cuda_status(cudaMemsetAsync(r.d_state.ptr, 0, RV_CARRIER_STATE_WORDS * 4, c->stream), "state clear");
    // fast mode: the tiled receivers' banded tap matrices for the tensor cores
    if (!st && c->fast && r.tile_cols != 0 && r.d_lerped.ptr) {
        r.tc_chunks = fine_tc_chunks(p.fine.taps, r.tile_period, (uint32_t)(fc / fd), (uint32_t)rem, (uint32_t)fd);
        st = r.d_tc.alloc(fine_tc_table_elements(r.tile_period, r.tc_chunks));
        if (!st)
            st = launch_fine_tc_tables(c->stream, r.d_lerped.ptr, p.fine.taps, r.period, r.tile_period, (uint32_t)(fc / fd),
                                       (uint32_t)rem, (uint32_t)fd, r.tc_chunks, r.d_tc.ptr);
    }
    if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "receiver setup");
    if (st) {
        r.d_taps.release();
        r.d_lerped.release();
        r.d_tc.release();
        r.d_fine.release();
        r.d_det.release();
        r.d_weights.release();
        r.d_state.release();
        return st;
    }
    {
        const uint32_t nw = (p.demod.channels == 2u && p.demod.pilot_taps != 0u)
                                ? stereo_weight_floats(p.demod.audio_taps, p.demod.pilot_taps)
                                : mono_weight_floats(p.demod.audio_taps);
        c->weights_cap = std::max<uint32_t>(c->weights_cap, (nw + 31u) & ~31u);
    }
    c->rx.push_back(std::move(r));
    c->table_dirty = true;
    if (id) *id = (uint32_t)(c->rx.size() - 1u);
    return clear_error();
}

int32_t rv_chain_run(rv_chain* c, const void* samples, uint64_t count, int32_t where) {
    if (c == nullptr || (samples == nullptr && count > 0)) return set_error_fmt(RV_ERR_INVALID, "rv_chain_run: NULL");
    if (count > c->config.max_run_samples)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_run: %llu samples exceed max_run_samples %u",
                             (unsigned long long)count, c->config.max_run_samples);
    if (count == 0) return clear_error();
    // this run's slot was last used two runs ago: hand that run's audio over
    if (int32_t st = collect_slot(c, S(c))) return st;
    const auto host_start = std::chrono::steady_clock::now();
    const rv_grid_params& g = c->config.grid;
    const bool plain = c->config.mode == RV_CHAIN_PLAIN;
    const uint8_t* src = static_cast<const uint8_t*>(samples);
    const uint64_t first_sample = c->samples_in;
    const uint64_t first_block = c->next_block;
    // the impulse excision lags the newest sample and the channelizer reads
    // only what it has finished (Graph::on_block, core/engine/graph.cpp:5025-5052)
    const rv_excision_plan* excision = plan_excision(c, first_sample, count);
    const uint64_t limit = excision ? std::min<uint64_t>(first_sample + count, excision->cleaned_end)
                                    : first_sample + count;
    uint32_t blocks = 0;
    if (limit > first_block * g.decimation) blocks = (uint32_t)((limit - 1u) / g.decimation - first_block + 1u);
    const uint64_t last_block = first_block + blocks - 1u;  // meaningful when blocks > 0
    mark(c, 0);
    // a captured run launches the coarse kernel inside its graph
    c->captured_run = !plain && c->graph && c->fused && blocks > 0 && !c->rx.empty();
    rv_coarse_params coarse{};
    int32_t st = plain ? coarse_plain(c, first_sample, src, count, where, first_block, blocks, excision)
                       : coarse_batched(c, first_sample, src, count, where, first_block, blocks,
                                        c->captured_run ? &coarse : nullptr, excision);
    if (st) return st;
    if (!c->captured_run) mark(c, 2);
    c->samples_in += count;
    c->next_block += blocks;
    c->stats.blocks += blocks;
    c->run_index += 1;
    if (blocks == 0 || c->rx.empty()) {
        if ((st = spectrum_frame(c, first_block, blocks))) return st;
        mark(c, 3);
        mark(c, 4);
        mark(c, 5);
        if (!pipelined(c) || S(c).sums_pending) {
            if ((st = cuda_status(cudaStreamSynchronize(c->stream), "run sync"))) return st;
            fe_collect(c, S(c));
            collect_marks(c);
        }
        return clear_error();
    }
    if (!plain && c->table_dirty)
        if ((st = upload_table(c))) return st;  // (a captured run whose table moved captures again)

    // ---- per-receiver cursors (DemodStage::record) and work lists
    std::vector<WorkItem> fine_items, carrier_items, unit_items;
    SpanTable rx_spans;
    if (!plain) {
        rx_spans.runs.assign(c->rx.size(), RxRun{});
        rx_spans.det_prefix.assign(c->rx.size() + 1u, 0u);
        rx_spans.audio_prefix.assign(c->rx.size() + 1u, 0u);
    }
    std::vector<FineUnit> units;
    std::vector<FineTile> tiles;
    struct TileSpan { uint32_t rx; uint64_t first, count; };
    std::vector<TileSpan> tile_spans;
    uint64_t tile_cost_total = 0;
    uint32_t fine_window = 0;
    uint64_t unit_cost_total = 0;
    struct UnitSpan { uint32_t rx, first, count; uint64_t cost_per_item; };
    std::vector<UnitSpan> unit_spans;
    uint64_t audio_floats = 0;
    struct Span { uint64_t fine_first, fine_count, det_first, det_count, audio_first, audio_count; };
    std::vector<Span> spans(c->rx.size());
    for (size_t ri = 0; ri < c->rx.size(); ++ri) {
        Receiver& r = c->rx[ri];
        const rv_vrx_plan_info& p = r.plan;
        const uint64_t fc = (uint64_t)p.channel_rate, fd = (uint64_t)p.demod_rate, dec = p.demod.decimation;
        if (!r.started) {
            const uint64_t needed = first_block + p.fine.taps - 1u;
            r.first_output = lowest_output_for(needed, fc, fd);
            r.next_output = r.first_output;
            r.next_audio = (r.first_output + r.fine_history + dec - 1u) / dec;
            r.started = true;
        }
        Span& s = spans[ri];
        memset(&s, 0, sizeof s);
        const uint64_t limit = highest_output_for(last_block, fc, fd);
        if (limit + 1u > r.next_output) {
            s.fine_first = r.next_output;
            s.fine_count = limit + 1u - r.next_output;
        }
        const uint64_t fine_end = s.fine_first + s.fine_count;
        if (s.fine_count) {
            const uint64_t det_from = std::max<uint64_t>(s.fine_first, r.first_output + r.det_history);
            if (fine_end > det_from) {
                s.det_first = det_from;
                s.det_count = fine_end - det_from;
            }
            r.next_output = fine_end;
        }
        if (r.next_output > r.first_output) {
            const uint64_t audio_limit = (r.next_output - 1u) / dec;
            if (audio_limit + 1u > r.next_audio) {
                s.audio_first = r.next_audio;
                s.audio_count = audio_limit + 1u - r.next_audio;
                r.next_audio += s.audio_count;
            }
        }
        r.run_audio_offset = audio_floats;
        r.run_audio_frames = s.audio_count;
        audio_floats += s.audio_count * p.demod.channels;
        if (!plain) {
            if (r.tile_cols != 0) {
                if (s.fine_count) {
                    tile_spans.push_back(TileSpan{(uint32_t)ri, s.fine_first, s.fine_count});
                    tile_cost_total += s.fine_count * p.fine.taps;
                }
            } else if (r.max_unit_item != 0) {
                const uint32_t before = (uint32_t)unit_items.size();
                push_fine_items(unit_items, (uint32_t)ri, r, s.fine_first, s.fine_count, r.max_unit_item);
                const uint32_t added = (uint32_t)unit_items.size() - before;
                if (added) {
                    unit_spans.push_back(UnitSpan{(uint32_t)ri, before, added, (uint64_t)r.max_unit_item * p.fine.taps});
                    unit_cost_total += s.fine_count * p.fine.taps;
                }
            } else {
                fine_window = std::max(fine_window, push_fine_items(fine_items, (uint32_t)ri, r, s.fine_first,
                                                                    s.fine_count, r.max_fine_item));
            }
            if (s.fine_count && p.carrier.power != 0) {
                carrier_items.push_back(WorkItem{(uint32_t)ri, (uint32_t)s.fine_count, s.fine_first, r.carrier_reset ? 1u : 0u});
                r.carrier_reset = false;
            }
            RxRun& run = rx_spans.runs[ri];
            if (!is_complex_demod(p.demod.mode)) {
                run.det_first = s.det_first;
                run.det_count = (uint32_t)s.det_count;
            }
            run.audio_first = s.audio_first;
            run.audio_count = (uint32_t)s.audio_count;
            run.audio_out = r.run_audio_offset;
            rx_spans.det_prefix[ri + 1u] = rx_spans.det_prefix[ri] + (run.det_count + r.max_det_item - 1u) / r.max_det_item;
            rx_spans.audio_prefix[ri + 1u] =
                rx_spans.audio_prefix[ri] + (run.audio_count + r.max_audio_item - 1u) / r.max_audio_item;
        }
    }
    if (S(c).audio_dev.count < audio_floats + 1)
        if ((st = S(c).audio_dev.alloc(audio_floats + 1 + audio_floats / 4))) return st;

    if (plain) {
        // the reference's recording: fine [+ carrier] + demod per receiver
        // (profiling books the whole receiver loop as fine_ms)
        for (size_t ri = 0; ri < c->rx.size(); ++ri) {
            Receiver& r = c->rx[ri];
            const Span& s = spans[ri];
            const rv_vrx_plan_info& p = r.plan;
            const uint32_t chan_base = p.placement.channel * c->chan_blocks;
            // fine dispatches small enough for the kernel's 32-bit recurrence
            const uint64_t rem = (uint64_t)(p.channel_rate % p.demod_rate);
            const uint64_t per = rem == 0 ? s.fine_count : std::max<uint64_t>(1, (0xFFFFFFFFull - (uint64_t)p.demod_rate) / rem);
            for (uint64_t done = 0; done < s.fine_count;) {
                const uint32_t n = (uint32_t)std::min<uint64_t>({s.fine_count - done, per, (uint64_t)r.fine_mask + 1u});
                rv_vrx_fine_block fb;
                if ((st = rv_fine_block(&p, chan_base, c->chan_blocks - 1u, r.fine_mask, s.fine_first + done, n, &fb))) return st;
                if ((st = rv_vrx_fine(c->stream, &p.fine, &fb.params, c->channel.ptr, c->channel.count, r.d_taps.ptr,
                                      r.d_taps.count, c->nco.ptr, c->nco.count, r.d_fine.ptr, r.d_fine.count)))
                    return st;
                c->stats.launches += 1;
                done += n;
            }
            if (s.fine_count && p.carrier.power != 0) {
                rv_vrx_carrier_params cp;
                if ((st = rv_carrier_block(&p, r.fine_mask, s.fine_first, (uint32_t)s.fine_count, r.carrier_reset, 0.0f, &cp)))
                    return st;
                if ((st = rv_vrx_carrier(c->stream, &p.carrier, &cp, c->nco.ptr, c->nco.count, r.d_fine.ptr,
                                         r.d_fine.count, r.d_state.ptr)))
                    return st;
                r.carrier_reset = false;
                c->stats.launches += 1;
            }
            if (s.audio_count) {
                rv_vrx_demod_block db;
                if ((st = rv_demod_block(&p, r.fine_mask, s.audio_first, (uint32_t)s.audio_count, &db))) return st;
                if ((st = rv_vrx_demod(c->stream, &p.demod, &db.params, r.d_fine.ptr, r.d_fine.count, r.d_weights.ptr,
                                       r.d_weights.count, S(c).audio_dev.ptr + r.run_audio_offset,
                                       s.audio_count * p.demod.channels)))
                    return st;
                c->stats.launches += 1;
            }
        }
        mark(c, 3);
        mark(c, 4);
    } else {
        // cost-balanced units and tiles: about four per SM
        {
            int sms = 0, dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            const uint64_t tile_target =
                std::max<uint64_t>(1, tile_cost_total / ((uint64_t)c->tiles_per_sm * (uint64_t)std::max(sms, 1)));
            for (const TileSpan& ts : tile_spans) push_tiles(tiles, ts.rx, c->rx[ts.rx], ts.first, ts.count, tile_target);
            // largest first, so the last tiles to start are the short ones (a
            // tensor-core tile costs its K chunks whatever its rows)
            auto tile_cost = [&](const FineTile& t) {
                const Receiver& r = c->rx[t.rx];
                return r.tc_chunks != 0 ? (uint64_t)r.tc_chunks : (uint64_t)t.rows * t.width * r.plan.fine.taps;
            };
            std::stable_sort(tiles.begin(), tiles.end(),
                             [&](const FineTile& x, const FineTile& y) { return tile_cost(x) > tile_cost(y); });
            const uint64_t target = std::max<uint64_t>(1, unit_cost_total / (uint64_t)(4 * std::max(sms, 1)));
            for (const UnitSpan& us : unit_spans) {
                const uint32_t per = (uint32_t)std::max<uint64_t>(1, target / std::max<uint64_t>(1, us.cost_per_item));
                for (uint32_t k = 0; k < us.count; k += per)
                    units.push_back(FineUnit{us.rx, us.first + k, std::min(per, us.count - k), c->rx[us.rx].table_rows});
            }
        }
        if (c->graph) {
            rx_spans.det_total = rx_spans.det_prefix.back();
            rx_spans.audio_total = rx_spans.audio_prefix.back();
            if ((st = run_captured(c, coarse, fine_items, carrier_items, rx_spans, unit_items, units, tiles, fine_window)))
                return st;
        } else {
        // unit items sit after the per-item lists; units index into that tail
        rx_spans.det_total = rx_spans.det_prefix.back();
        rx_spans.audio_total = rx_spans.audio_prefix.back();
        if ((st = upload_spans(c, rx_spans))) return st;
        const size_t unit_base = fine_items.size() + carrier_items.size();
        for (FineUnit& u : units) u.first_item += (uint32_t)unit_base;
        const size_t total = unit_base + unit_items.size();
        if ((st = S(c).items_host.reserve(total + 1 + total / 2))) return st;  // headroom: no re-pinning per run
        if (S(c).queues.count == 0)
            if ((st = S(c).queues.alloc(1))) return st;
        if ((st = cuda_status(cudaMemsetAsync(S(c).queues.ptr, 0, sizeof(Queues), c->stream), "queue reset"))) return st;
        if (S(c).items_dev.count < total + 1)
            if ((st = S(c).items_dev.alloc(total + 1 + total / 4))) return st;
        WorkItem* h = S(c).items_host.ptr;
        size_t at = 0;
        for (auto* list : {&fine_items, &carrier_items, &unit_items}) {
            if (!list->empty()) memcpy(h + at, list->data(), list->size() * sizeof(WorkItem));
            at += list->size();
        }
        if ((st = cuda_status(cudaMemcpyAsync(S(c).items_dev.ptr, h, total * sizeof(WorkItem), cudaMemcpyHostToDevice,
                                              c->stream),
                              "work list upload")))
            return st;
        if (!units.empty()) {
            if ((st = S(c).units_host.reserve(units.size() + units.size() / 2 + 1))) return st;
            if (S(c).units_dev.count < units.size())
                if ((st = S(c).units_dev.alloc(units.size() + units.size() / 2 + 1))) return st;
            memcpy(S(c).units_host.ptr, units.data(), units.size() * sizeof(FineUnit));
            if ((st = cuda_status(cudaMemcpyAsync(S(c).units_dev.ptr, S(c).units_host.ptr, units.size() * sizeof(FineUnit),
                                                  cudaMemcpyHostToDevice, c->stream),
                                  "unit upload")))
                return st;
        }
        if (!tiles.empty()) {
            if ((st = S(c).tiles_host.reserve(tiles.size() + tiles.size() / 2 + 1))) return st;
            if (S(c).tiles_dev.count < tiles.size())
                if ((st = S(c).tiles_dev.alloc(tiles.size() + tiles.size() / 2 + 1))) return st;
            memcpy(S(c).tiles_host.ptr, tiles.data(), tiles.size() * sizeof(FineTile));
            if ((st = cuda_status(cudaMemcpyAsync(S(c).tiles_dev.ptr, S(c).tiles_host.ptr, tiles.size() * sizeof(FineTile),
                                                  cudaMemcpyHostToDevice, c->stream),
                                  "tile upload")))
                return st;
        }
        if (c->hoisted) {
            // the plain recording with the detector hoisted: fine [+ carrier]
            // per receiver through the per-dispatch kernels, then the detector
            // and the audio per receiver through the batched kernels, each
            // launch given only its receiver's items
            const size_t nrx = c->rx.size();
            for (size_t ri = 0; ri < nrx; ++ri) {
                Receiver& r = c->rx[ri];
                const Span& sp = spans[ri];
                const rv_vrx_plan_info& p = r.plan;
                const uint32_t chan_base = p.placement.channel * c->chan_blocks;
                const uint64_t rem = (uint64_t)(p.channel_rate % p.demod_rate);
                const uint64_t per = rem == 0 ? sp.fine_count : std::max<uint64_t>(1, (0xFFFFFFFFull - (uint64_t)p.demod_rate) / rem);
                for (uint64_t done = 0; done < sp.fine_count;) {
                    const uint32_t n = (uint32_t)std::min<uint64_t>({sp.fine_count - done, per, (uint64_t)r.fine_mask + 1u});
                    rv_vrx_fine_block fb;
                    if ((st = rv_fine_block(&p, chan_base, c->chan_blocks - 1u, r.fine_mask, sp.fine_first + done, n, &fb)))
                        return st;
                    if ((st = rv_vrx_fine(c->stream, &p.fine, &fb.params, c->channel.ptr, c->channel.count, r.d_taps.ptr,
                                          r.d_taps.count, c->nco.ptr, c->nco.count, r.d_fine.ptr, r.d_fine.count)))
                        return st;
                    c->stats.launches += 1;
                    done += n;
                }
            }
            for (const WorkItem& it : carrier_items) {  // item: receiver, count, first fine output, reset flag (out)
                Receiver& r = c->rx[it.rx];
                rv_vrx_carrier_params cp;
                if ((st = rv_carrier_block(&r.plan, r.fine_mask, it.first, it.count, it.out != 0u, 0.0f, &cp))) return st;
                if ((st = rv_vrx_carrier(c->stream, &r.plan.carrier, &cp, c->nco.ptr, c->nco.count, r.d_fine.ptr,
                                         r.d_fine.count, r.d_state.ptr)))
                    return st;
                c->stats.launches += 1;
            }
            mark(c, 3);
            // receiver ri's prefix sums: zero up to ri, its count after (the
            // kernels' search then finds ri for every item)
            const size_t stride = 2u * (nrx + 1u);
            std::vector<uint32_t> hp(nrx * stride, 0u);
            for (size_t ri = 0; ri < nrx; ++ri) {
                const uint32_t nd = rx_spans.det_prefix[ri + 1u] - rx_spans.det_prefix[ri];
                const uint32_t na = rx_spans.audio_prefix[ri + 1u] - rx_spans.audio_prefix[ri];
                for (size_t k = ri + 1u; k <= nrx; ++k) {
                    hp[ri * stride + k] = nd;
                    hp[ri * stride + nrx + 1u + k] = na;
                }
            }
            if (c->hoisted_prefix.count < hp.size())
                if ((st = c->hoisted_prefix.alloc(hp.size()))) return st;
            if ((st = cuda_status(cudaMemcpyAsync(c->hoisted_prefix.ptr, hp.data(), hp.size() * sizeof(uint32_t),
                                                  cudaMemcpyHostToDevice, c->stream),
                                  "hoisted prefix upload")))
                return st;
            const RxRun* runs = reinterpret_cast<const RxRun*>(S(c).spans_dev.ptr);
            for (size_t ri = 0; ri < nrx; ++ri) {
                const uint32_t* pre = c->hoisted_prefix.ptr + ri * stride;
                const uint32_t nd = hp[ri * stride + nrx], na = hp[ri * stride + 2u * nrx + 1u];
                if (nd) {
                    if ((st = cuda_status(cudaMemsetAsync(&S(c).queues.ptr->detect, 0, sizeof(uint32_t), c->stream),
                                          "queue reset")))
                        return st;
                    if ((st = launch_detect_batched(c->stream, c->rx_table.ptr, SpanList{runs, pre, (uint32_t)nrx, 0u}, nd,
                                                    kDetWindow, &S(c).queues.ptr->detect)))
                        return st;
                    c->stats.launches += 1;
                }
                if (na) {
                    if ((st = cuda_status(cudaMemsetAsync(&S(c).queues.ptr->audio, 0, sizeof(uint32_t), c->stream),
                                          "queue reset")))
                        return st;
                    if ((st = launch_audio_batched(c->stream, c->rx_table.ptr, SpanList{runs, pre + nrx + 1u, (uint32_t)nrx, 1u},
                                                   na, S(c).audio_dev.ptr, kDetWindow, c->weights_cap,
                                                   &S(c).queues.ptr->audio)))
                        return st;
                    c->stats.launches += 1;
                }
            }
            mark(c, 4);
        } else {
            const WorkItem* d = S(c).items_dev.ptr;
            const float2* chan = reinterpret_cast<const float2*>(c->channel.ptr);
            if ((st = c->fast ? launch_fine_tc(c->stream, c->rx_table.ptr, S(c).tiles_dev.ptr, (uint32_t)tiles.size(), chan,
                                               &S(c).queues.ptr->tiles, nullptr, c->tc_status.ptr)
                              : launch_fine_tiles(c->stream, c->rx_table.ptr, S(c).tiles_dev.ptr, (uint32_t)tiles.size(), chan,
                                                  c->tile_shared, &S(c).queues.ptr->tiles)))
                return st;
            if ((st = launch_fine_units(c->stream, c->rx_table.ptr, S(c).items_dev.ptr, S(c).units_dev.ptr,
                                        (uint32_t)units.size(), chan, c->unit_budget, &S(c).queues.ptr->units)))
                return st;
            const uint32_t window = std::min<uint32_t>(kFineWindow, (fine_window + 255u) & ~255u);
            if ((st = launch_fine_batched(c->stream, c->rx_table.ptr, d, (uint32_t)fine_items.size(), chan, window,
                                          &S(c).queues.ptr->fine)))
                return st;
            d += fine_items.size();
            if ((st = launch_carrier_batched(c->stream, c->rx_table.ptr, d, (uint32_t)carrier_items.size()))) return st;
            d += carrier_items.size();
            mark(c, 3);
            SpanList det_list, audio_list;
            span_lists(c, (uint32_t)c->rx.size(), &det_list, &audio_list);
            if ((st = launch_detect_batched(c->stream, c->rx_table.ptr, det_list, rx_spans.det_total, kDetWindow,
                                            &S(c).queues.ptr->detect, nullptr, c->fast)))
                return st;
            if ((st = launch_audio_batched(c->stream, c->rx_table.ptr, audio_list, rx_spans.audio_total, S(c).audio_dev.ptr,
                                           kDetWindow, c->weights_cap, &S(c).queues.ptr->audio, nullptr, c->fast)))
                return st;
            mark(c, 4);
            c->stats.launches += (rx_spans.det_total ? 1 : 0) + (rx_spans.audio_total ? 1 : 0) + (fine_items.empty() ? 0 : 1) +
                                 (units.empty() ? 0 : 1) + (carrier_items.empty() ? 0 : 1) + (tiles.empty() ? 0 : 1);
            c->stats.work_items += total + rx_spans.det_total + rx_spans.audio_total + tiles.size();
        }
        }
    }

    c->stats.host_ms +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_start).count();
    if ((st = spectrum_frame(c, first_block, blocks))) return st;
    // ---- audio back to the host (the reference's readback copies), into the
    // slot; handed to the receivers now, or when the slot comes round again
    RunSlot& sl = S(c);
    sl.audio_floats = audio_floats;
    sl.parts.resize(c->rx.size());
    for (size_t i = 0; i < c->rx.size(); ++i) sl.parts[i] = {c->rx[i].run_audio_offset, c->rx[i].run_audio_frames};
    if (audio_floats > 0) {
        if ((st = sl.audio_host.reserve(audio_floats + audio_floats / 4))) return st;
        if ((st = cuda_status(cudaMemcpyAsync(sl.audio_host.ptr, sl.audio_dev.ptr, audio_floats * sizeof(float),
                                              cudaMemcpyDeviceToHost, c->stream),
                              "audio readback")))
            return st;
    }
    mark(c, 5);
    if ((st = cuda_status(cudaEventRecord(sl.done, c->stream), "run event"))) return st;
    sl.pending = true;
    c->stats.runs += 1;
    if (pipelined(c)) {
        c->cur ^= 1u;  // the next run prepares the other slot while this one executes
        return clear_error();
    }
    if ((st = collect_slot(c, sl))) return st;
    collect_marks(c);
    return clear_error();
}

namespace {

// Mean device time of the fine tiles of `rxs` over one run of `outputs[i]`
// fine outputs each (cut `per_sm` tiles per SM, the list repeated until it
// fills the GPU `fill` times), shared memory `shared` float2s a CTA.
int32_t time_tiles(rv_chain* c, const std::vector<uint32_t>& rxs, const std::vector<uint64_t>& outputs,
                   uint32_t per_sm, uint32_t shared, uint32_t fill, DeviceArray<FineTile>& d_tiles,
                   DeviceArray<uint32_t>& queue, cudaEvent_t e0, cudaEvent_t e1, double* ms) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t cost = 0;
    for (size_t i = 0; i < rxs.size(); ++i) cost += outputs[i] * c->rx[rxs[i]].plan.fine.taps;
    const uint64_t target = std::max<uint64_t>(1, cost / ((uint64_t)per_sm * (uint64_t)std::max(sms, 1)));
    std::vector<FineTile> one, tiles;
    for (size_t i = 0; i < rxs.size(); ++i) push_tiles(one, rxs[i], c->rx[rxs[i]], 0, outputs[i], target);
    if (one.empty()) return set_error_fmt(RV_ERR_INVALID, "rv_chain_autotune: no tiles to time");
    while (tiles.size() < (size_t)fill * (size_t)std::max(sms, 1)) tiles.insert(tiles.end(), one.begin(), one.end());
    std::stable_sort(tiles.begin(), tiles.end(), [&](const FineTile& x, const FineTile& y) {
        return (uint64_t)x.rows * x.width * c->rx[x.rx].plan.fine.taps > (uint64_t)y.rows * y.width * c->rx[y.rx].plan.fine.taps;
    });
    if (d_tiles.count < tiles.size())
        if (int32_t st = d_tiles.alloc(tiles.size())) return st;
    if (int32_t st = cuda_status(cudaMemcpy(d_tiles.ptr, tiles.data(), tiles.size() * sizeof(FineTile), cudaMemcpyHostToDevice),
                                 "autotune tiles"))
        return st;
    const float2* chan = reinterpret_cast<const float2*>(c->channel.ptr);
    const uint32_t n = (uint32_t)tiles.size();
    constexpr int kReps = 3;
    for (int rep = -1; rep < kReps; ++rep) {  // one untimed launch first
        if (rep == 0)
            if (int32_t st = cuda_status(cudaEventRecord(e0, c->stream), "autotune event")) return st;
        if (int32_t st = cuda_status(cudaMemsetAsync(queue.ptr, 0, sizeof(uint32_t), c->stream), "autotune queue"))
            return st;
        if (int32_t st = launch_fine_tiles(c->stream, c->rx_table.ptr, d_tiles.ptr, n, chan, shared, queue.ptr)) return st;
    }
    if (int32_t st = cuda_status(cudaEventRecord(e1, c->stream), "autotune event")) return st;
    if (int32_t st = cuda_status(cudaEventSynchronize(e1), "autotune sync")) return st;
    float elapsed = 0.0f;
    if (int32_t st = cuda_status(cudaEventElapsedTime(&elapsed, e0, e1), "autotune time")) return st;
    *ms = elapsed / kReps;
    return RV_OK;
}

}  // namespace

extern "C" int32_t rv_chain_autotune(rv_chain* c, uint32_t run_samples, rv_chain_tune_report* report) {
    if (c == nullptr || report == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_autotune: NULL argument");
    memset(report, 0, sizeof *report);
    if (c->config.mode != RV_CHAIN_BATCHED || c->fast || c->hoisted)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_chain_autotune: tunes the batched chain's fine tiles");
    if (run_samples == 0) return set_error_fmt(RV_ERR_INVALID, "rv_chain_autotune: run_samples is 0");
    for (const Receiver& r : c->rx)
        if (r.started)
            return set_error_fmt(RV_ERR_INVALID, "rv_chain_autotune: tune before the first run (its rings are written)");
    if (int32_t st = cuda_status(cudaStreamSynchronize(c->stream), "autotune sync")) return st;
    // one run's fine outputs per receiver, and the classes: receivers of the
    // same rates, taps and pattern period share their shapes
    const uint64_t blocks = run_samples / c->config.grid.decimation;
    std::map<std::tuple<int64_t, int64_t, uint32_t, uint32_t>, std::vector<uint32_t>> classes;
    std::vector<uint32_t> tiled;
    std::vector<uint64_t> outputs(c->rx.size(), 0);
    for (uint32_t i = 0; i < (uint32_t)c->rx.size(); ++i) {
        const Receiver& r = c->rx[i];
        if (r.tile_cols == 0) continue;
        outputs[i] = blocks * (uint64_t)r.plan.demod_rate / (uint64_t)r.plan.channel_rate;
        if (outputs[i] == 0) continue;
        tiled.push_back(i);
        classes[std::make_tuple(r.plan.channel_rate, r.plan.demod_rate, r.plan.fine.taps, r.period)].push_back(i);
    }
    if (tiled.empty()) return clear_error();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    DeviceArray<FineTile> d_tiles;
    DeviceArray<uint32_t> queue;
    int32_t st = cuda_status(cudaEventCreate(&e0), "autotune event");
    if (!st) st = cuda_status(cudaEventCreate(&e1), "autotune event");
    if (!st) st = queue.alloc(1);
    auto all_outputs = [&](const std::vector<uint32_t>& rxs) {
        std::vector<uint64_t> o;
        for (uint32_t i : rxs) o.push_back(outputs[i]);
        return o;
    };
    auto max_shared = [&]() {
        uint32_t m = 0;
        for (uint32_t i : tiled) m = std::max(m, c->rx[i].tile_shared);
        return m;
    };
    // the rule's shapes, 4 tiles per SM: the default. A launch's shared
    // memory is the largest shape's, so the rule's largest bounds every
    // candidate (a larger one would take CTAs per SM from every tile)
    double default_ms = 0.0, tuned_ms = 0.0;
    const uint32_t launch_shared = max_shared();
    std::vector<TileShape> rule_shapes(c->rx.size());
    for (uint32_t i : tiled) {
        const Receiver& r = c->rx[i];
        TileShape& t = rule_shapes[i];
        t.cols = r.tile_cols, t.block = r.tile_block, t.rows = r.tile_rows, t.buffers = r.tile_buffers;
        t.seg = r.tile_seg, t.stride = r.tile_stride, t.period = r.tile_period, t.shared = r.tile_shared;
        t.row_step = r.row_step;
    }
    if (!st) st = upload_table(c);
    if (!st) st = time_tiles(c, tiled, all_outputs(tiled), 4, launch_shared, 1, d_tiles, queue, e0, e1, &default_ms);
    // each class: every shape within the launch's shared memory, timed on
    // the class's tiles repeated to fill the GPU four times over
    const uint32_t budgets[1] = {launch_shared};
    for (auto it = classes.begin(); !st && it != classes.end(); ++it) {
        const std::vector<uint32_t>& members = it->second;
        Receiver& r0 = c->rx[members[0]];
        const uint64_t fc = (uint64_t)r0.plan.channel_rate, fd = (uint64_t)r0.plan.demod_rate;
        std::vector<TileShape> shapes, candidates;
        for (uint32_t b : budgets) tile_shapes(r0, fc, fd, b, shapes);
        for (const TileShape& sh : shapes) {
            bool seen = false;
            for (const TileShape& o : candidates) seen = seen || o.same(sh);
            if (!seen) candidates.push_back(sh);
        }
        const TileShape rule = rule_shapes[members[0]];
        const TileShape* best = nullptr;
        double best_ms = 0.0;
        for (const TileShape& sh : candidates) {
            for (uint32_t i : members) set_tile_shape(c->rx[i], sh);
            double ms = 0.0;
            if ((st = upload_table(c))) break;
            if ((st = time_tiles(c, members, all_outputs(members), 4, launch_shared, 4, d_tiles, queue, e0, e1, &ms))) break;
            ++report->shapes_timed;
            // the rule's shape unless another is clearly faster
            const double bias = sh.same(rule) ? 0.97 : 1.0;
            if (best == nullptr || ms * bias < best_ms) {
                best = &sh;
                best_ms = ms * bias;
            }
        }
        if (st) break;
        for (uint32_t i : members) set_tile_shape(c->rx[i], *best);
        ++report->classes;
        if (!best->same(rule)) ++report->classes_changed;
    }
    // the tuned shapes together: kept only when the whole run is faster
    if (!st) st = upload_table(c);
    double together_ms = 0.0;
    if (!st) st = time_tiles(c, tiled, all_outputs(tiled), 4, launch_shared, 1, d_tiles, queue, e0, e1, &together_ms);
    if (!st && !(together_ms < default_ms)) {
        for (uint32_t i : tiled) set_tile_shape(c->rx[i], rule_shapes[i]);
        report->classes_changed = 0;
        report->shapes_reverted = 1;
        st = upload_table(c);
    }
    // tiles per SM, on the shapes kept
    uint32_t per_sm = 4;
    double best_ms = 0.0;
    for (uint32_t k : {2u, 4u, 8u}) {
        double ms = 0.0;
        if (st || (st = time_tiles(c, tiled, all_outputs(tiled), k, launch_shared, 1, d_tiles, queue, e0, e1, &ms))) break;
        if (k == 2u || ms < best_ms) {
            best_ms = ms;
            per_sm = k;
        }
    }
    tuned_ms = best_ms;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    d_tiles.release();
    queue.release();
    // the timed launches wrote the fine rings: back to a stream start
    c->tile_shared = std::max(max_shared(), launch_shared);
    for (uint32_t i : tiled) {
        Receiver& r = c->rx[i];
        if (!st) st = cuda_status(cudaMemsetAsync(r.d_fine.ptr, 0, r.d_fine.count * sizeof(rv_cf32), c->stream), "fine clear");
    }
    if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "autotune sync");
    c->table_dirty = true;
    if (st) return st;
    c->tiles_per_sm = per_sm;
    report->tiles_per_sm = per_sm;
    report->default_ms = default_ms;
    report->tuned_ms = tuned_ms;
    report->receivers = (uint32_t)tiled.size();
    return clear_error();
}

int32_t rv_chain_capture_graph(rv_chain* c) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_capture_graph: NULL");
    if (c->config.mode != RV_CHAIN_BATCHED || c->hoisted)
        return set_error_fmt(RV_ERR_UNSUPPORTED,
                             "rv_chain_capture_graph: a plain or hoisted chain records one launch per stage per "
                             "receiver; only the batched chain runs from a graph");
    if (!c->fused)
        return set_error_fmt(RV_ERR_UNSUPPORTED,
                             "rv_chain_capture_graph: no fused channelizer kernel for M=%u T=%u D=%u; this chain's "
                             "channelizer runs as per-run dispatches",
                             c->config.grid.channels, c->config.grid.taps_per_branch, c->config.grid.decimation);
    c->graph = true;
    return clear_error();
}

int32_t rv_chain_set_front_end(rv_chain* c, int32_t dc_removal, int32_t iq_correction, uint32_t lag) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_front_end: NULL");
    if (lag == 0 || lag > 64) return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_front_end: lag %u outside [1, 64]", lag);
    if (pipelined(c) && lag < 2)
        return set_error_fmt(RV_ERR_INVALID,
                             "rv_chain_set_front_end: a pipelined chain reads a run's moments back two runs later; "
                             "lag must be at least 2");
    c->fe_dc = dc_removal != 0;
    c->fe_iq = iq_correction != 0;
    c->fe_lag = lag;
    return clear_error();
}

int32_t rv_chain_front_end_estimate(rv_chain* c, rv_front_end* out) {
    if (c == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_front_end_estimate: NULL");
    if (int32_t st = collect_all(c)) return st;
    *out = c->fe;
    return clear_error();
}

int32_t rv_chain_set_impulse_excision(rv_chain* c, int32_t on, double threshold_db, double max_width_seconds) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_impulse_excision: NULL");
    if (int32_t st = rv_chain_drain(c)) return st;
    if (!on) {
        c->ex_on = false;
        return clear_error();
    }
    if (!std::isfinite(threshold_db) || threshold_db < -100.0 || threshold_db > 100.0)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_impulse_excision: threshold %g dB", threshold_db);
    if (!std::isfinite(max_width_seconds) || max_width_seconds <= 0.0)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_impulse_excision: max width %g s", max_width_seconds);
    rv_excision_config cfg{};
    if (int32_t st = rv_design_excision(c->config.rate, max_width_seconds, &cfg)) return st;
    rv_excision_rings rings{};
    if (int32_t st = rv_size_excision_rings(&cfg, c->config.max_run_samples, pipelined(c) ? 2u : 1u, c->raw_mask, &rings))
        return st;
    const uint64_t cap = (uint64_t)c->raw_mask + 1u;
    int32_t st = RV_OK;
    if (c->config.mode == RV_CHAIN_BATCHED && c->clean.count < cap) {
        st = c->clean.alloc(cap);
        if (!st) st = cuda_status(cudaMemsetAsync(c->clean.ptr, 0, cap * sizeof(rv_cf32), c->stream), "ring clear");
    }
    if (!st && c->ex_seg_power.count != (uint64_t)rings.seg_mask + 1u) {
        st = c->ex_seg_power.alloc((uint64_t)rings.seg_mask + 1u);
        if (!st) st = c->ex_seg_level.alloc((uint64_t)rings.seg_mask + 1u);
    }
    if (!st && c->ex_flags.count != (uint64_t)rings.flag_mask + 1u) st = c->ex_flags.alloc((uint64_t)rings.flag_mask + 1u);
    if (!st && c->ex_removed.count != (uint64_t)rings.removed_mask + 1u)
        st = c->ex_removed.alloc((uint64_t)rings.removed_mask + 1u);
    if (!st && c->ex_counters.count == 0) st = c->ex_counters.alloc(RV_EXCISE_COUNTERS);
    if (!st)
        st = cuda_status(cudaMemsetAsync(c->ex_counters.ptr, 0, RV_EXCISE_COUNTERS * sizeof(uint32_t), c->stream),
                         "excision counters");
    if (st) return st;
    c->ex_cfg = cfg;
    c->ex_rings = rings;
    c->ex_threshold = rv_excision_threshold(threshold_db);
    if (int32_t e = rv_excision_cursor_init(&c->ex_cursor, &cfg, c->raw_mask, &rings, c->ex_threshold)) return e;
    c->ex_on = true;
    c->ex_was_on = false;
    if (c->config.mode == RV_CHAIN_BATCHED && !c->ex_clean) {
        c->ex_clean = true;
        c->ex_converted_end = ~0ull;  // the clean ring holds nothing of this stream yet
    }
    return clear_error();
}

int32_t rv_chain_excision_counters(rv_chain* c, uint64_t* out) {
    if (c == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_excision_counters: NULL");
    if (int32_t st = rv_chain_drain(c)) return st;
    if (c->ex_counters.count) {
        uint32_t d[RV_EXCISE_COUNTERS] = {0, 0, 0, 0};
        if (int32_t st = cuda_status(cudaMemcpy(d, c->ex_counters.ptr, sizeof d, cudaMemcpyDeviceToHost),
                                     "excision counters"))
            return st;
        if (int32_t st = cuda_status(cudaMemsetAsync(c->ex_counters.ptr, 0, sizeof d, c->stream), "excision counters"))
            return st;
        for (int k = 0; k < 3; ++k) c->ex_totals[k] += d[k];
    }
    for (int k = 0; k < 3; ++k) out[k] = c->ex_totals[k];
    out[3] = c->ex_examined;
    return clear_error();
}

int32_t rv_chain_set_spectrum(rv_chain* c, uint32_t transform, rv_detector* detector) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_spectrum: NULL");
    if (int32_t st = collect_all(c)) return st;
    if (transform == 0) {
        c->spec_n = 0;
        c->detector = nullptr;
        return clear_error();
    }
    if (!is_pow2(transform) || transform < 8 || transform > 2048)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_spectrum: transform %u must be a power of two in [8, 2048]",
                             transform);
    if ((uint64_t)transform > c->chan_blocks)
        return set_error_fmt(RV_ERR_INVALID, "rv_chain_set_spectrum: %u points exceed the %u-block channel ring",
                             transform, c->chan_blocks);
    const rv_grid_params& g = c->config.grid;
    std::vector<float> window;
    std::vector<rv_cf32> tw;
    if (int32_t st = build_window(transform, g.taps_per_branch, c->config.attenuation_db, window)) return st;
    if (int32_t st = build_twiddle_table(transform, tw)) return st;
    int32_t st = c->spec_window.alloc(window.size());
    if (!st) st = c->spec_twiddles.alloc(tw.size());
    if (!st) st = c->spec_frame.alloc((uint64_t)g.channels * transform / 2u);
    if (!st) st = cuda_status(cudaMemcpyAsync(c->spec_window.ptr, window.data(), window.size() * 4, cudaMemcpyHostToDevice,
                                              c->stream), "spectrum window upload");
    if (!st) st = cuda_status(cudaMemcpyAsync(c->spec_twiddles.ptr, tw.data(), tw.size() * 8, cudaMemcpyHostToDevice,
                                              c->stream), "spectrum twiddle upload");
    if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "spectrum setup");
    if (st) return st;
    c->spec_n = transform;
    c->detector = detector;
    c->spec_recorded = false;
    return clear_error();
}

int32_t rv_chain_read_spectrum(rv_chain* c, float* out, uint64_t capacity, uint64_t* bins, uint64_t* start,
                               uint64_t* count, uint64_t* sequence) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_read_spectrum: NULL");
    if (int32_t st = collect_all(c)) return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(c->stream), "spectrum read")) return st;
    const uint64_t n = c->spec_n ? (uint64_t)c->config.grid.channels * c->spec_n / 2u : 0u;
    if (bins) *bins = c->spec_recorded ? n : 0u;
    if (start) *start = c->spec_start;
    if (count) *count = c->spec_count;
    if (sequence) *sequence = c->spec_sequence;
    if (out && c->spec_recorded && n)
        if (int32_t st = cuda_status(cudaMemcpy(out, c->spec_frame.ptr, std::min(capacity, n) * sizeof(float),
                                                cudaMemcpyDeviceToHost),
                                     "spectrum read"))
            return st;
    return clear_error();
}

int32_t rv_chain_drain(rv_chain* c) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_drain: NULL");
    if (int32_t st = collect_all(c)) return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(c->stream), "rv_chain_drain")) return st;
    if (c->copy_stream)
        if (int32_t st = cuda_status(cudaStreamSynchronize(c->copy_stream), "rv_chain_drain")) return st;
    if (c->fast) {  // a bounded tensor-core wait that ran out
        uint32_t timeouts = 0;
        if (int32_t st = cuda_status(cudaMemcpy(&timeouts, c->tc_status.ptr, sizeof timeouts, cudaMemcpyDeviceToHost),
                                     "rv_chain_drain"))
            return st;
        if (timeouts)
            return set_error_fmt(RV_ERR_TIMEOUT, "rv_chain_drain: %u fine-stage CTAs gave up waiting on the tensor cores",
                                 timeouts);
    }
    return clear_error();
}

int32_t rv_chain_receiver_info(const rv_chain* c, uint32_t id, rv_vrx_plan_info* info, uint64_t* audio_frames,
                               uint64_t* first_audio) {
    if (c == nullptr || id >= c->rx.size()) return set_error_fmt(RV_ERR_INVALID, "rv_chain_receiver_info: no receiver %u", id);
    if (int32_t st = collect_all(const_cast<rv_chain*>(c))) return st;  // runs in flight first
    const Receiver& r = c->rx[id];
    if (info) *info = r.plan;
    if (audio_frames) *audio_frames = r.audio_frames_total;
    if (first_audio) *first_audio = r.next_audio - r.audio_frames_total;
    return clear_error();
}

int32_t rv_chain_read_audio(rv_chain* c, uint32_t id, float* dst, uint64_t capacity, uint64_t* written) {
    if (c == nullptr || id >= c->rx.size()) return set_error_fmt(RV_ERR_INVALID, "rv_chain_read_audio: no receiver %u", id);
    if (int32_t st = collect_all(c)) return st;  // runs in flight first
    Receiver& r = c->rx[id];
    const uint64_t n = std::min<uint64_t>(capacity, r.audio.size());
    if (dst && n) memcpy(dst, r.audio.data(), n * sizeof(float));
    r.audio.erase(r.audio.begin(), r.audio.begin() + n);
    if (written) *written = n;
    return clear_error();
}

int32_t rv_chain_get_stats(const rv_chain* c, rv_chain_stats* stats) {
    if (c == nullptr || stats == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_get_stats: NULL");
    if (int32_t st = collect_all(const_cast<rv_chain*>(c))) return st;  // runs in flight first
    *stats = c->stats;
    return clear_error();
}

int32_t rv_chain_receiver_rings(const rv_chain* c, uint32_t id, const rv_cf32** fine, const float** det, uint32_t* mask) {
    if (c == nullptr || id >= c->rx.size()) return set_error_fmt(RV_ERR_INVALID, "rv_chain_receiver_rings: no receiver %u", id);
    const Receiver& r = c->rx[id];
    if (fine) *fine = r.d_fine.ptr;
    if (det) *det = c->config.mode == RV_CHAIN_BATCHED ? r.d_det.ptr : nullptr;
    if (mask) *mask = r.fine_mask;
    return clear_error();
}

int32_t rv_chain_channel_ring(const rv_chain* c, const rv_cf32** ring, uint32_t* ring_blocks) {
    if (c == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_chain_channel_ring: NULL");
    if (ring) *ring = c->channel.ptr;
    if (ring_blocks) *ring_blocks = c->chan_blocks;
    return clear_error();
}

}  // extern "C"
