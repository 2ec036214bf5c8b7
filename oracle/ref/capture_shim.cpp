// extern "C" access to the reference's own capture segment writer
// (core/capture/writer.cpp SegmentWriter, recover_open_segments), compiled
// from the reference sources into oracle/_ref/libcapref.so. Test
// infrastructure only: the capture tests drive it and the library's writer
// with the same blocks and compare the files they leave.
//
// The reference writes from its own thread. Each write here waits (bounded)
// until that thread has written the block, so that annotations and gain
// changes land between the same blocks as in a synchronous writer.
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "core/capture/writer.h"

using namespace revenant;

namespace {

struct Handle {
    std::shared_ptr<std::atomic<std::int64_t>> now;
    std::unique_ptr<capture::SegmentWriter> writer;
    std::uint64_t fed_bytes = 0;
};

source::SampleFormat format_of(int f) {
    switch (f) {
        case 1: return source::SampleFormat::Cs8;
        case 2: return source::SampleFormat::Cs16;
        case 3: return source::SampleFormat::Cs24;
        default: return source::SampleFormat::Cu8;
    }
}

}  // namespace

extern "C" {

void* refcap_open(const char* root, std::uint64_t max_bytes, double max_seconds, std::uint64_t retention_bytes,
                  std::int64_t retention_age_ns, std::uint64_t epoch, int recover, const char* hw, std::int64_t now_ns) {
    auto* h = new Handle;
    h->now = std::make_shared<std::atomic<std::int64_t>>(now_ns);
    capture::WriterConfig c;
    c.root = root;
    c.max_segment_bytes = max_bytes;
    c.max_segment_seconds = max_seconds;
    c.retention_bytes = retention_bytes;
    c.retention_max_age_ns = retention_age_ns;
    c.queue_blocks = 1 << 16;
    c.stream_epoch = epoch;
    c.hw = hw ? hw : "";
    c.recover_on_start = recover != 0;
    auto now = h->now;
    c.now_ns = [now] { return now->load(); };
    h->writer = std::make_unique<capture::SegmentWriter>(c);
    if (!h->writer->start()) {
        delete h;
        return nullptr;
    }
    return h;
}

int refcap_write(void* handle, std::uint64_t first, std::int64_t anchor, std::int64_t rate, std::int64_t center,
                 std::uint64_t count, std::uint64_t dropped, int format, const void* bytes, std::uint64_t nbytes) {
    auto* h = static_cast<Handle*>(handle);
    source::SourceBlock b;
    b.stamp = dsp::BlockTimestamp{first, anchor, rate};
    b.format = format_of(format);
    b.sample_count = count;
    b.bytes = std::span<const std::byte>(static_cast<const std::byte*>(bytes), nbytes);
    b.dropped_before = dropped;
    h->writer->consume(b, center);
    h->fed_bytes += nbytes;
    for (int i = 0; i < 20000; ++i) {  // at most 10 s
        const auto s = h->writer->stats();
        if (s.bytes_written >= h->fed_bytes) return 0;
        if (!s.last_error.empty()) return -2;
        std::this_thread::sleep_for(std::chrono::microseconds(500));
    }
    return -1;
}

void refcap_set_gain(void* handle, int has, double gain) {
    static_cast<Handle*>(handle)->writer->set_gain_db(has ? std::optional<double>(gain) : std::nullopt);
}

void refcap_set_clock(void* handle, std::int64_t now_ns) { static_cast<Handle*>(handle)->now->store(now_ns); }

void refcap_annotate(void* handle, std::uint64_t start, std::uint64_t count, std::int64_t lo, std::int64_t hi,
                     double confidence, double peak_db, double snr_db, int has_track, std::uint64_t track_id,
                     const char* family) {
    capture::Annotation a;
    a.sample_count = count;
    a.freq_lower = lo;
    a.freq_upper = hi;
    a.confidence = confidence;
    a.peak_db = peak_db;
    a.snr_db = snr_db;
    a.family = family ? family : "";
    static_cast<Handle*>(handle)->writer->add_annotation(
        start, a, has_track ? std::optional<std::uint64_t>(track_id) : std::nullopt);
}

// {segments_written, bytes_written, segments_deleted, annotations_discarded,
//  annotations_merged_late, retained_bytes, stream_epoch}
void refcap_stats(void* handle, std::uint64_t out[7]) {
    auto* h = static_cast<Handle*>(handle);
    const auto s = h->writer->stats();
    const std::uint64_t v[7] = {s.segments_written, s.bytes_written, s.segments_deleted, s.annotations_discarded,
                                s.annotations_merged_late, s.retained_bytes, h->writer->stream_epoch()};
    std::memcpy(out, v, sizeof v);
}

void refcap_close(void* handle) {
    auto* h = static_cast<Handle*>(handle);
    h->writer->stop();
    delete h;
}

int refcap_recover(const char* root, std::uint64_t out[3]) {
    auto r = capture::recover_open_segments(root);
    if (!r) return -1;
    out[0] = r->recovered;
    out[1] = r->removed_empty;
    out[2] = r->failures.size();
    return 0;
}

}  // extern "C"
