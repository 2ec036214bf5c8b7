// The rolling capture's on-disk segments (core/capture/format.h,
// core/capture/writer.cpp), so that a capture replays through the chain.
//
// A segment is a SigMF recording: <root>/<YYYY-MM-DD>/<stem>.sigmf-data, the
// raw samples in the source's own format, and <stem>.sigmf-meta, a JSON
// sidecar written when the segment closes. A segment is homogeneous and
// gapless. Before a block is written the open segment closes when the block
// does not continue it (writer.cpp SegmentWriter::process, in this order):
// samples were lost ("loss"), the index went backwards ("stop"; a new run of
// the source, so a new stream epoch), the format, the rate or the centre
// changed ("format", "rate", "retune"), or the block would take the segment
// past its byte limit, or the segment already holds its seconds limit
// ("size"). Blocks are never split.
//
// While open, the data file is <stem>.open.sigmf-data with <stem>.open.revenant
// beside it (rate, format, anchor, dropped count, gain, hw), so that a segment
// whose writer died can still be closed by rv_capture_recover.
//
//   stem = "rev-" UTC yyyymmddThhmmss.fffZ of the first sample
//          "-" centre Hz "-" stream epoch (16 hex digits) "-" first index
//
// Annotations (the detector's tracks, generator "revenant-detect") are filed
// by stream index: the part inside the open segment goes into its meta at
// close, a part inside a closed segment is merged into that meta at once, and
// what lies past the open segment waits for the next.
//
// The reference writes from a thread behind a bounded queue; here a block is
// written when it is handed over, so nothing is dropped for a full queue and
// the caller picks the thread.
#include <dirent.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <deque>
#include <random>
#include <string>
#include <vector>

#include "revenant_gb300.h"

namespace rv {
int32_t set_error_fmt(int32_t code, const char* fmt, ...);
int32_t clear_error();
}  // namespace rv

namespace {

using rv::set_error_fmt;

constexpr const char* kDetectGenerator = "revenant-detect";
constexpr size_t kClosedIndexLimit = 1024;

// ---- time ------------------------------------------------------------------

struct Civil {
    int64_t year;
    unsigned month, day, hour, minute, second;
    int64_t nanos;
};

// Days since 1970-01-01 <-> proleptic Gregorian dates (the era-based
// conversions of H. Hinnant's "chrono-compatible low-level date algorithms").
void civil_from_days(int64_t z, int64_t& y, unsigned& m, unsigned& d) {
    z += 719468;
    const int64_t era = (z >= 0 ? z : z - 146096) / 146097;
    const unsigned doe = (unsigned)(z - era * 146097);
    const unsigned yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
    y = (int64_t)yoe + era * 400;
    const unsigned doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
    const unsigned mp = (5 * doy + 2) / 153;
    d = doy - (153 * mp + 2) / 5 + 1;
    m = mp < 10 ? mp + 3 : mp - 9;
    if (m <= 2) ++y;
}

int64_t days_from_civil(int64_t y, unsigned m, unsigned d) {
    y -= m <= 2;
    const int64_t era = (y >= 0 ? y : y - 399) / 400;
    const unsigned yoe = (unsigned)(y - era * 400);
    const unsigned doy = (153 * (m > 2 ? m - 3 : m + 9) + 2) / 5 + d - 1;
    const unsigned doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
    return era * 146097 + (int64_t)doe - 719468;
}

Civil to_civil(int64_t ns) {
    const int64_t per_day = 86400ll * 1000000000ll;
    int64_t days = ns / per_day, rem = ns % per_day;
    if (rem < 0) {
        rem += per_day;
        --days;
    }
    Civil c;
    civil_from_days(days, c.year, c.month, c.day);
    const int64_t secs = rem / 1000000000ll;
    c.nanos = rem % 1000000000ll;
    c.hour = (unsigned)(secs / 3600);
    c.minute = (unsigned)((secs / 60) % 60);
    c.second = (unsigned)(secs % 60);
    return c;
}

// BlockTimestamp::wall_clock_ns (core/dsp/types.h): whole seconds and the
// remainder converted separately so index * 1e9 never overflows.
int64_t wall_clock_ns(uint64_t index, int64_t anchor, int64_t rate) {
    if (rate <= 0) return anchor;
    const uint64_t r = (uint64_t)rate;
    const int64_t whole = (int64_t)(index / r), rem = (int64_t)(index % r);
    return anchor + whole * 1000000000ll + (rem * 1000000000ll) / rate;
}

std::string iso_datetime(int64_t ns) {
    const Civil c = to_civil(ns);
    char buf[64];
    snprintf(buf, sizeof buf, "%04lld-%02u-%02uT%02u:%02u:%02u.%09lldZ", (long long)c.year, c.month, c.day, c.hour,
             c.minute, c.second, (long long)c.nanos);
    return buf;
}

std::string day_of(int64_t ns) {
    const Civil c = to_civil(ns);
    char buf[24];
    snprintf(buf, sizeof buf, "%04lld-%02u-%02u", (long long)c.year, c.month, c.day);
    return buf;
}

int64_t system_now_ns() {
    timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    return (int64_t)ts.tv_sec * 1000000000ll + ts.tv_nsec;
}

// ---- formats ---------------------------------------------------------------

bool known_format(int32_t f) {
    return f == RV_FORMAT_CU8 || f == RV_FORMAT_CS8 || f == RV_FORMAT_CS16 || f == RV_FORMAT_CS24;
}
uint32_t bytes_per_sample(int32_t f) { return f == RV_FORMAT_CS24 ? 6u : f == RV_FORMAT_CS16 ? 4u : 2u; }
// SigMF core:datatype (writer.cpp sigmf_datatype).
const char* sigmf_datatype(int32_t f) {
    return f == RV_FORMAT_CS24 ? "ci24_le" : f == RV_FORMAT_CS16 ? "ci16_le" : f == RV_FORMAT_CS8 ? "ci8" : "cu8";
}
int32_t format_from_datatype(const std::string& t) {
    if (t == "ci24_le") return RV_FORMAT_CS24;
    if (t == "ci16_le") return RV_FORMAT_CS16;
    if (t == "ci8") return RV_FORMAT_CS8;
    if (t == "cu8") return RV_FORMAT_CU8;
    return -1;
}
// The side file names formats the way the source does
// (core/source/capabilities.h format_name).
const char* source_name(int32_t f) {
    return f == RV_FORMAT_CS24 ? "cs24" : f == RV_FORMAT_CS16 ? "cs16" : f == RV_FORMAT_CS8 ? "cs8" : "cu8";
}
int32_t format_from_source_name(const std::string& n) {
    if (n == "cs24") return RV_FORMAT_CS24;
    if (n == "cs16") return RV_FORMAT_CS16;
    if (n == "cs8") return RV_FORMAT_CS8;
    if (n == "cu8") return RV_FORMAT_CU8;
    return -1;
}

// ---- text ------------------------------------------------------------------

// Shortest round-trip decimal of a double (what std::format "{}" prints);
// JSON has no spelling for a non-finite number, so those become null.
std::string number_text(double v) {
    if (!std::isfinite(v)) return "null";
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof buf, v);
    return std::string(buf, r.ptr);
}

// A JSON builder over a string: separators from an open/first/after-key
// state, and the string escapes the reference's meta uses (\" \\ \n \r \t,
// other control bytes as \u00XX).
class Json {
  public:
    void open_object() { sep(); out_ += '{'; first_ = true; }
    void close_object() { out_ += '}'; first_ = false; }
    void open_array() { sep(); out_ += '['; first_ = true; }
    void close_array() { out_ += ']'; first_ = false; }
    void key(const std::string& k) { sep(); literal(k); out_ += ':'; after_key_ = true; }
    void str(const std::string& s) { sep(); literal(s); }
    void u64(uint64_t v) { sep(); out_ += std::to_string((unsigned long long)v); }
    void i64(int64_t v) { sep(); out_ += std::to_string((long long)v); }
    void f64(double v) { sep(); out_ += number_text(v); }
    void boolean(bool v) { sep(); out_ += v ? "true" : "false"; }
    std::string take() { return std::move(out_); }

  private:
    void sep() {
        if (after_key_) {
            after_key_ = false;
            return;
        }
        if (!first_) out_ += ',';
        first_ = false;
    }
    void literal(const std::string& s) {
        out_ += '"';
        for (char ch : s) {
            switch (ch) {
                case '"': out_ += "\\\""; break;
                case '\\': out_ += "\\\\"; break;
                case '\n': out_ += "\\n"; break;
                case '\r': out_ += "\\r"; break;
                case '\t': out_ += "\\t"; break;
                default:
                    if ((unsigned char)ch < 0x20) {
                        char b[8];
                        snprintf(b, sizeof b, "\\u%04x", (unsigned)(unsigned char)ch);
                        out_ += b;
                    } else {
                        out_ += ch;
                    }
            }
        }
        out_ += '"';
    }
    std::string out_;
    bool first_ = true, after_key_ = false;
};

bool write_file(const std::string& path, const std::string& text) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(text.data(), 1, text.size(), f) == text.size();
    return fclose(f) == 0 && ok;
}

// Write beside, then rename over: a reader never sees half a meta.
bool replace_file(const std::string& path, const std::string& text) {
    const std::string tmp = path + ".tmp";
    if (!write_file(tmp, text)) return false;
    if (rename(tmp.c_str(), path.c_str()) != 0) {
        remove(tmp.c_str());
        return false;
    }
    return true;
}

bool read_text(const std::string& path, std::string& out) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    char buf[4096];
    size_t n;
    out.clear();
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

bool file_size(const std::string& path, uint64_t& size) {
    struct stat sb;
    if (stat(path.c_str(), &sb) != 0) return false;
    size = (uint64_t)sb.st_size;
    return true;
}

bool exists(const std::string& path) {
    struct stat sb;
    return stat(path.c_str(), &sb) == 0;
}

bool is_dir(const std::string& path) {
    struct stat sb;
    return stat(path.c_str(), &sb) == 0 && S_ISDIR(sb.st_mode);
}

bool make_dirs(const std::string& path) {
    if (path.empty() || is_dir(path)) return true;
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos && slash > 0 && !make_dirs(path.substr(0, slash))) return false;
    return mkdir(path.c_str(), 0755) == 0 || errno == EEXIST;
}

bool ends_with(const std::string& s, const std::string& tail) {
    return s.size() > tail.size() && s.compare(s.size() - tail.size(), tail.size(), tail) == 0;
}

std::vector<std::string> entries(const std::string& dir) {
    std::vector<std::string> out;
    DIR* d = opendir(dir.c_str());
    if (d == nullptr) return out;
    while (dirent* e = readdir(d))
        if (e->d_name[0] != '.') out.push_back(e->d_name);
    closedir(d);
    std::sort(out.begin(), out.end());
    return out;
}

bool parse_i64(const std::string& t, int64_t& v) {
    if (t.empty()) return false;
    const auto r = std::from_chars(t.data(), t.data() + t.size(), v);
    return r.ec == std::errc{} && r.ptr == t.data() + t.size();
}

bool parse_u64(const std::string& t, uint64_t& v, int base = 10) {
    if (t.empty()) return false;
    const auto r = std::from_chars(t.data(), t.data() + t.size(), v, base);
    return r.ec == std::errc{} && r.ptr == t.data() + t.size();
}

bool parse_f64(const std::string& t, double& v) {
    if (t.empty()) return false;
    const auto r = std::from_chars(t.data(), t.data() + t.size(), v);
    return r.ec == std::errc{} && r.ptr == t.data() + t.size();
}

// ---- stems -----------------------------------------------------------------

struct StemFields {
    int64_t center = 0;
    uint64_t stream_epoch = 0, first_index = 0;
    int64_t start_ns = 0;
};

std::string make_stem(uint64_t first, int64_t center, uint64_t epoch, int64_t start_ns) {
    const Civil c = to_civil(start_ns);
    char buf[160];
    snprintf(buf, sizeof buf, "rev-%04lld%02u%02uT%02u%02u%02u.%03lldZ-%lld-%016llx-%llu", (long long)c.year, c.month,
             c.day, c.hour, c.minute, c.second, (long long)(c.nanos / 1000000), (long long)center,
             (unsigned long long)epoch, (unsigned long long)first);
    return buf;
}

// writer.cpp parse_stem: the fields split at the first dash and the last two,
// so a negative centre parses.
bool parse_stem(const std::string& stem, StemFields& out) {
    if (stem.compare(0, 4, "rev-") != 0) return false;
    const std::string rest = stem.substr(4);
    const size_t a = rest.find('-'), c = rest.rfind('-');
    if (a == std::string::npos || c == a) return false;
    const size_t b = rest.rfind('-', c - 1);
    if (b == std::string::npos || b <= a) return false;
    const std::string time = rest.substr(0, a), epoch = rest.substr(b + 1, c - b - 1);
    if (!parse_i64(rest.substr(a + 1, b - a - 1), out.center) || epoch.size() != 16 ||
        !parse_u64(epoch, out.stream_epoch, 16) || !parse_u64(rest.substr(c + 1), out.first_index))
        return false;
    if (time.size() != 20 || time[8] != 'T' || time[15] != '.' || time[19] != 'Z') return false;
    int64_t y, mo, d, h, mi, s, ms;
    if (!parse_i64(time.substr(0, 4), y) || !parse_i64(time.substr(4, 2), mo) || !parse_i64(time.substr(6, 2), d) ||
        !parse_i64(time.substr(9, 2), h) || !parse_i64(time.substr(11, 2), mi) || !parse_i64(time.substr(13, 2), s) ||
        !parse_i64(time.substr(16, 3), ms))
        return false;
    if (mo < 1 || mo > 12 || d < 1) return false;
    static const unsigned kDays[] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
    const bool leap = (y % 4 == 0 && y % 100 != 0) || y % 400 == 0;
    if (d > (int64_t)(kDays[mo - 1] + (mo == 2 && leap ? 1 : 0))) return false;
    const int64_t days = days_from_civil(y, (unsigned)mo, (unsigned)d);
    out.start_ns = ((days * 86400 + h * 3600 + mi * 60 + s) * 1000 + ms) * 1000000ll;
    return true;
}

// ---- meta ------------------------------------------------------------------

struct SegmentInfo {
    uint64_t stream_epoch = 0, first_index = 0, sample_count = 0, dropped_before = 0;
    int64_t epoch_anchor_ns = 0, rate = 0, center = 0;
    int32_t format = RV_FORMAT_CU8;
    uint64_t end_index() const { return first_index + sample_count; }
    int64_t start_ns() const { return wall_clock_ns(first_index, epoch_anchor_ns, rate); }
};

struct Entry {
    rv_capture_annotation a;  // sample_count clipped to the segment
    uint64_t sample_start = 0;  // relative to the segment's first sample
    std::string generator = kDetectGenerator;
};

struct MetaFields {
    SegmentInfo info;
    std::string close_reason, hw;
    bool has_gain = false;
    double gain_db = 0;
    std::vector<Entry> annotations;
};

std::string field_text(const char* chars, size_t cap) { return std::string(chars, strnlen(chars, cap)); }

// The meta, key for key in the reference's order (writer.cpp render_meta).
std::string render_meta(const MetaFields& f) {
    const SegmentInfo& i = f.info;
    Json j;
    j.open_object();
    j.key("global");
    j.open_object();
    j.key("core:datatype"), j.str(sigmf_datatype(i.format));
    j.key("core:sample_rate"), j.i64(i.rate);
    j.key("core:version"), j.str("1.2.0");
    j.key("core:num_channels"), j.u64(1);
    j.key("core:recorder"), j.str("Revenant " RV_CAPTURE_RECORDER_VERSION);
    j.key("core:hw"), j.str(f.hw);
    j.key("core:extensions");
    j.open_array();
    j.open_object();
    j.key("name"), j.str("revenant");
    j.key("version"), j.str("1.1.0");
    j.key("optional"), j.boolean(true);
    j.close_object();
    j.close_array();
    j.key("revenant:stream_epoch"), j.u64(i.stream_epoch);
    j.key("revenant:first_index"), j.u64(i.first_index);
    j.key("revenant:epoch_anchor_ns"), j.i64(i.epoch_anchor_ns);
    j.key("revenant:dropped_before"), j.u64(i.dropped_before);
    j.key("revenant:close_reason"), j.str(f.close_reason);
    if (f.has_gain) j.key("revenant:gain_db"), j.f64(f.gain_db);
    j.close_object();
    j.key("captures");
    j.open_array();
    j.open_object();
    j.key("core:sample_start"), j.u64(0);
    j.key("core:frequency"), j.i64(i.center);
    j.key("core:datetime"), j.str(iso_datetime(i.start_ns()));
    j.close_object();
    j.close_array();
    j.key("annotations");
    j.open_array();
    for (const Entry& e : f.annotations) {
        const std::string family = field_text(e.a.family, sizeof e.a.family);
        j.open_object();
        j.key("core:sample_start"), j.u64(e.sample_start);
        j.key("core:sample_count"), j.u64(e.a.sample_count);
        j.key("core:freq_lower_edge"), j.i64(e.a.freq_lower);
        j.key("core:freq_upper_edge"), j.i64(e.a.freq_upper);
        j.key("core:label"), j.str(family.empty() ? "signal" : family);
        j.key("core:generator"), j.str(e.generator);
        j.key("revenant:confidence"), j.f64(e.a.confidence);
        j.key("revenant:peak_db"), j.f64(e.a.peak_db);
        j.key("revenant:snr_db"), j.f64(e.a.snr_db);
        if (!family.empty()) j.key("revenant:family"), j.str(family);
        if (e.a.has_track_id) j.key("revenant:track_id"), j.u64(e.a.track_id);
        j.close_object();
    }
    j.close_array();
    j.close_object();
    return j.take() + "\n";
}

// writer.cpp render_side: what recovery needs to interpret an open segment.
std::string render_side(const SegmentInfo& i, const MetaFields& f) {
    std::string hw = f.hw;
    for (char& ch : hw)
        if (ch == '\n' || ch == '\r') ch = ' ';
    std::string out = "rate=" + std::to_string((long long)i.rate) + "\nformat=" + source_name(i.format) +
                      "\nanchor_ns=" + std::to_string((long long)i.epoch_anchor_ns) +
                      "\ndropped_before=" + std::to_string((unsigned long long)i.dropped_before) + "\n";
    if (f.has_gain) out += "gain_db=" + number_text(f.gain_db) + "\n";
    return out + "hw=" + hw + "\n";
}

// The number or string after "key": in a meta (each global key at most once).
bool json_field(const std::string& text, const char* key, std::string& out) {
    const std::string k = std::string("\"") + key + "\":";
    size_t at = text.find(k);
    if (at == std::string::npos) return false;
    at += k.size();
    if (at < text.size() && text[at] == '"') {
        size_t end = at + 1;
        while (end < text.size() && text[end] != '"') end += text[end] == '\\' ? 2 : 1;
        if (end >= text.size()) return false;
        out = text.substr(at + 1, end - at - 1);
        return true;
    }
    size_t end = at;
    while (end < text.size() && text[end] != ',' && text[end] != '}' && text[end] != ']') ++end;
    out = text.substr(at, end - at);
    return !out.empty();
}

// The part of [start, start + count) inside [first, end); a zero-length
// annotation is a point and belongs to the segment holding it.
bool clip(uint64_t start, uint64_t count, uint64_t first, uint64_t end, uint64_t& low, uint64_t& n) {
    if (count == 0) {
        low = start, n = 0;
        return start >= first && start < end;
    }
    low = std::max(start, first);
    const uint64_t high = std::min(start + count, end);
    n = high > low ? high - low : 0;
    return high > low;
}

uint64_t draw_epoch() {
    std::random_device dev;
    const uint64_t v = ((uint64_t)dev() << 32) ^ (uint64_t)dev();
    const uint64_t masked = v & 0x7FFFFFFFFFFFFFFFull;  // a signed 64-bit JSON reader reads it exactly
    return masked == 0 ? 1 : masked;
}

struct Pending {
    uint64_t start;
    rv_capture_annotation a;
};

struct Closed {
    MetaFields meta;
    std::string meta_path;
};

struct Retained {
    std::string data, meta, order_key;
    uint64_t bytes = 0;
    int64_t start_ns = 0;
};

// Meta first, then data, then the day directory if that left it empty
// (writer.cpp remove_pair).
bool remove_pair(const Retained& r) {
    if (remove(r.meta.c_str()) != 0 && exists(r.meta)) return false;
    if (remove(r.data.c_str()) != 0 && exists(r.data)) return false;
    const std::string dir = r.data.substr(0, r.data.find_last_of('/'));
    if (entries(dir).empty()) rmdir(dir.c_str());
    return true;
}

}  // namespace

struct rv_capture_writer {
    std::string root, hw;
    rv_capture_config config{};
    int64_t clock_ns = 0;  // 0 = the system clock
    bool has_gain = false;
    double gain_db = 0;

    // the open segment
    bool open = false;
    SegmentInfo info;
    MetaFields open_meta;  // gain and hw as of the open
    std::string dir, stem;
    uint64_t bytes = 0;
    FILE* out = nullptr;

    bool have_last = false;
    uint64_t last_end = 0;
    std::vector<Pending> pending;
    std::deque<Closed> closed;
    std::vector<Retained> retained;
    rv_capture_writer_stats stats{};

    int64_t now() const { return clock_ns != 0 ? clock_ns : system_now_ns(); }
};

namespace {

std::string base_of(const rv_capture_writer* w) { return w->dir + "/" + w->stem; }

void index_existing(rv_capture_writer* w) {
    w->retained.clear();
    for (const std::string& day : entries(w->root)) {
        const std::string dir = w->root + "/" + day;
        if (!is_dir(dir)) continue;
        for (const std::string& name : entries(dir)) {
            if (!ends_with(name, ".sigmf-meta")) continue;
            const std::string stem = name.substr(0, name.size() - 11);
            StemFields f;
            uint64_t data_bytes, meta_bytes;
            if (!parse_stem(stem, f) || !file_size(dir + "/" + stem + ".sigmf-data", data_bytes)) continue;
            Retained r;
            r.data = dir + "/" + stem + ".sigmf-data";
            r.meta = dir + "/" + name;
            r.bytes = data_bytes + (file_size(r.meta, meta_bytes) ? meta_bytes : 0);
            r.start_ns = f.start_ns;
            r.order_key = day + "/" + stem;
            w->retained.push_back(r);
        }
    }
    std::sort(w->retained.begin(), w->retained.end(),
              [](const Retained& a, const Retained& b) { return a.order_key < b.order_key; });
}

// writer.cpp apply_retention: the oldest closed segments go first while the
// closed ones plus the open one are over the byte budget, or while the oldest
// is older than the age limit.
void apply_retention(rv_capture_writer* w) {
    const rv_capture_config& c = w->config;
    if (c.retention_bytes == 0 && c.retention_max_age_ns <= 0) return;
    std::sort(w->retained.begin(), w->retained.end(),
              [](const Retained& a, const Retained& b) { return a.order_key < b.order_key; });
    uint64_t total = w->open ? w->bytes : 0;
    for (const Retained& r : w->retained) total += r.bytes;
    const int64_t now = w->now();
    size_t taken = 0;
    while (taken < w->retained.size()) {
        const Retained& oldest = w->retained[taken];
        const bool over = c.retention_bytes != 0 && total > c.retention_bytes;
        const bool old = c.retention_max_age_ns > 0 && now - oldest.start_ns > c.retention_max_age_ns;
        if (!over && !old) break;
        if (remove_pair(oldest)) {
            total -= std::min(total, oldest.bytes);
            w->stats.retained_bytes -= std::min(w->stats.retained_bytes, oldest.bytes);
            ++w->stats.segments_deleted;
        } else {
            ++w->stats.delete_failures;
        }
        ++taken;
    }
    w->retained.erase(w->retained.begin(), w->retained.begin() + (ptrdiff_t)taken);
}

int32_t close_segment(rv_capture_writer* w, const char* reason) {
    if (!w->open) return RV_OK;
    const bool flushed = fclose(w->out) == 0;
    w->out = nullptr;
    w->open = false;
    const std::string base = base_of(w);
    if (!flushed) return set_error_fmt(RV_ERR_INVALID, "capture: closing %s.open.sigmf-data failed", base.c_str());
    if (w->info.sample_count == 0) {
        remove((base + ".open.sigmf-data").c_str());
        remove((base + ".open.revenant").c_str());
        return RV_OK;
    }
    MetaFields meta = w->open_meta;
    meta.info = w->info;
    meta.close_reason = reason;
    const uint64_t first = w->info.first_index, end = w->info.end_index();
    std::vector<Pending> keep;
    for (Pending& p : w->pending) {
        uint64_t low, n;
        if (clip(p.start, p.a.sample_count, first, end, low, n)) {
            Entry e;
            e.a = p.a;
            e.a.sample_count = n;
            e.sample_start = low - first;
            meta.annotations.push_back(e);
        }
        // the rest carries on into the next segment
        const uint64_t stop = p.start + p.a.sample_count;
        if (stop > end || p.start >= end) {
            const uint64_t from = std::max(p.start, end);
            p.a.sample_count = stop > from ? stop - from : 0;
            p.start = from;
            keep.push_back(p);
        }
    }
    w->pending = std::move(keep);
    std::stable_sort(meta.annotations.begin(), meta.annotations.end(),
                     [](const Entry& a, const Entry& b) { return a.sample_start < b.sample_start; });
    const std::string meta_path = base + ".sigmf-meta";
    if (!write_file(meta_path, render_meta(meta))) {
        remove(meta_path.c_str());
        return set_error_fmt(RV_ERR_INVALID, "capture: cannot write %s", meta_path.c_str());
    }
    if (rename((base + ".open.sigmf-data").c_str(), (base + ".sigmf-data").c_str()) != 0)
        return set_error_fmt(RV_ERR_INVALID, "capture: cannot rename %s.open.sigmf-data", base.c_str());
    remove((base + ".open.revenant").c_str());
    uint64_t meta_bytes = 0;
    Retained r;
    r.data = base + ".sigmf-data";
    r.meta = meta_path;
    r.bytes = w->bytes + (file_size(meta_path, meta_bytes) ? meta_bytes : 0);
    r.start_ns = w->info.start_ns();
    r.order_key = w->dir.substr(w->dir.find_last_of('/') + 1) + "/" + w->stem;
    w->retained.push_back(r);
    w->closed.push_back(Closed{std::move(meta), meta_path});
    if (w->closed.size() > kClosedIndexLimit) w->closed.pop_front();
    ++w->stats.segments_written;
    w->stats.retained_bytes += r.bytes;
    apply_retention(w);
    return RV_OK;
}

int32_t open_segment(rv_capture_writer* w, const rv_capture_block& b, uint64_t dropped_before) {
    SegmentInfo& i = w->info;
    i = SegmentInfo{};
    i.stream_epoch = w->config.stream_epoch;
    i.first_index = b.first_index;
    i.epoch_anchor_ns = b.epoch_anchor_ns;
    i.rate = b.rate;
    i.center = b.center;
    i.format = b.format;
    i.dropped_before = dropped_before;
    w->open_meta = MetaFields{};
    w->open_meta.hw = w->hw;
    w->open_meta.has_gain = w->has_gain;
    w->open_meta.gain_db = w->gain_db;
    w->stem = make_stem(i.first_index, i.center, i.stream_epoch, i.start_ns());
    w->dir = w->root + "/" + day_of(i.start_ns());
    w->bytes = 0;
    if (!make_dirs(w->dir)) return set_error_fmt(RV_ERR_INVALID, "capture: cannot create %s", w->dir.c_str());
    // the side file goes down before the first sample
    const std::string base = base_of(w);
    if (!write_file(base + ".open.revenant", render_side(i, w->open_meta)))
        return set_error_fmt(RV_ERR_INVALID, "capture: cannot write %s.open.revenant", base.c_str());
    w->out = fopen((base + ".open.sigmf-data").c_str(), "wb");
    if (!w->out) return set_error_fmt(RV_ERR_INVALID, "capture: cannot create %s.open.sigmf-data", base.c_str());
    w->open = true;
    return RV_OK;
}

// A part that falls in a closed segment is merged into its meta now; the
// rest waits for the open segment's close (writer.cpp route_annotations).
void route(rv_capture_writer* w, uint64_t start, const rv_capture_annotation& a) {
    const uint64_t count = a.sample_count;
    const uint64_t tail = w->closed.empty() ? 0 : w->closed.back().meta.info.end_index();
    if (!w->closed.empty() && start < w->closed.front().meta.info.first_index) ++w->stats.annotations_discarded;
    for (Closed& c : w->closed) {
        const uint64_t first = c.meta.info.first_index, end = c.meta.info.end_index();
        if (end <= start) continue;
        if (!(first < start + count || first <= start)) break;
        uint64_t low, n;
        if (!clip(start, count, first, end, low, n)) continue;
        Entry e;
        e.a = a;
        e.a.sample_count = n;
        e.sample_start = low - first;
        if (!exists(c.meta_path)) {  // retention deleted it
            ++w->stats.annotations_discarded;
            continue;
        }
        c.meta.annotations.push_back(e);
        if (!replace_file(c.meta_path, render_meta(c.meta))) {
            c.meta.annotations.pop_back();
            ++w->stats.annotations_discarded;
            continue;
        }
        ++w->stats.annotations_merged_late;
    }
    const uint64_t stop = start + count;
    if (stop > tail || start >= tail) {
        const uint64_t from = std::max(start, tail);
        rv_capture_annotation rest = a;
        rest.sample_count = stop > from ? stop - from : 0;
        w->pending.push_back(Pending{from, rest});
    }
}

// writer.cpp recover_open_segments.
void recover(const std::string& root, uint32_t counts[3]) {
    counts[0] = counts[1] = counts[2] = 0;
    const std::string tail = ".open.sigmf-data";
    for (const std::string& day : entries(root)) {
        const std::string dir = root + "/" + day;
        if (!is_dir(dir)) continue;
        for (const std::string& name : entries(dir)) {
            if (!ends_with(name, tail)) continue;
            const std::string stem = name.substr(0, name.size() - tail.size()), base = dir + "/" + stem;
            StemFields f;
            std::string side;
            if (!parse_stem(stem, f) || !read_text(base + ".open.revenant", side)) {
                ++counts[2];
                continue;
            }
            MetaFields m;
            m.info.stream_epoch = f.stream_epoch;
            m.info.first_index = f.first_index;
            m.info.center = f.center;
            m.close_reason = "recovered";
            bool have_rate = false, have_format = false, have_anchor = false;
            for (size_t at = 0; at < side.size();) {
                size_t nl = side.find('\n', at);
                if (nl == std::string::npos) nl = side.size();
                const std::string line = side.substr(at, nl - at);
                at = nl + 1;
                const size_t eq = line.find('=');
                if (eq == std::string::npos) continue;
                const std::string k = line.substr(0, eq), v = line.substr(eq + 1);
                if (k == "rate") {
                    have_rate = parse_i64(v, m.info.rate) && m.info.rate > 0;
                } else if (k == "format") {
                    m.info.format = format_from_source_name(v);
                    have_format = m.info.format >= 0;
                } else if (k == "anchor_ns") {
                    have_anchor = parse_i64(v, m.info.epoch_anchor_ns);
                } else if (k == "dropped_before") {
                    parse_u64(v, m.info.dropped_before);
                } else if (k == "gain_db") {
                    m.has_gain = parse_f64(v, m.gain_db);
                } else if (k == "hw") {
                    m.hw = v;
                }
            }
            uint64_t size;
            if (!have_rate || !have_format || !have_anchor || !file_size(base + tail, size)) {
                ++counts[2];
                continue;
            }
            const uint64_t bps = bytes_per_sample(m.info.format), whole = size / bps * bps;
            // a partial sample is the tail of the write the process died in
            if (whole != size && truncate((base + tail).c_str(), (off_t)whole) != 0) {
                ++counts[2];
                continue;
            }
            if (whole == 0) {
                remove((base + tail).c_str());
                remove((base + ".open.revenant").c_str());
                ++counts[1];
                continue;
            }
            m.info.sample_count = whole / bps;
            // a meta already there is the complete one: the writer died between it and the rename
            if (!exists(base + ".sigmf-meta") && !write_file(base + ".sigmf-meta", render_meta(m))) {
                ++counts[2];
                continue;
            }
            if (rename((base + tail).c_str(), (base + ".sigmf-data").c_str()) != 0) {
                ++counts[2];
                continue;
            }
            remove((base + ".open.revenant").c_str());
            ++counts[0];
        }
    }
}

}  // namespace

extern "C" {

int32_t rv_capture_writer_open(const char* root, const rv_capture_config* config, const char* hw,
                               rv_capture_writer** out) {
    if (root == nullptr || config == nullptr || out == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_open: NULL argument");
    *out = nullptr;
    if (!(config->max_segment_seconds >= 0.0))
        return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_open: max_segment_seconds must be >= 0");
    if (!make_dirs(root)) return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_open: cannot create %s", root);
    auto* w = new rv_capture_writer;
    w->root = root;
    w->hw = hw ? hw : "";
    w->config = *config;
    if (config->recover_on_start) {
        uint32_t counts[3];
        recover(w->root, counts);
        w->stats.recovered = counts[0];
    }
    if (w->config.stream_epoch == 0) w->config.stream_epoch = draw_epoch();
    index_existing(w);
    for (const Retained& r : w->retained) w->stats.retained_bytes += r.bytes;
    *out = w;
    return rv::clear_error();
}

int32_t rv_capture_writer_write(rv_capture_writer* w, const rv_capture_block* block, const void* bytes,
                                uint64_t byte_count) {
    if (w == nullptr || block == nullptr || (bytes == nullptr && byte_count > 0))
        return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_write: NULL argument");
    const rv_capture_block& b = *block;
    if (!known_format(b.format))
        return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_capture_writer_write: format %d (cu8, cs8, cs16, cs24)", b.format);
    if (b.rate <= 0) return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_write: rate must be positive");
    if (byte_count != b.sample_count * bytes_per_sample(b.format))
        return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_write: %llu bytes for %llu %s samples",
                             (unsigned long long)byte_count, (unsigned long long)b.sample_count, source_name(b.format));
    const bool loss = b.dropped_before > 0;
    bool restarted = false;
    if (w->open) {
        const char* reason = nullptr;
        const uint64_t end = w->info.end_index();
        if (loss || b.first_index > end) {
            reason = "loss";
        } else if (b.first_index < end) {  // a new run of the source
            reason = "stop";
            restarted = true;
        } else if (b.format != w->info.format) {
            reason = "format";
        } else if (b.rate != w->info.rate) {
            reason = "rate";
        } else if (b.center != w->info.center) {
            reason = "retune";
        } else if (w->config.max_segment_bytes != 0 && w->bytes + byte_count > w->config.max_segment_bytes) {
            reason = "size";
        } else if (w->config.max_segment_seconds > 0.0 &&
                   (double)w->info.sample_count >= w->config.max_segment_seconds * (double)w->info.rate) {
            reason = "size";
        }
        if (reason)
            if (int32_t st = close_segment(w, reason)) return st;
    } else if (w->have_last && b.first_index < w->last_end) {
        restarted = true;
    }
    if (restarted) {
        w->config.stream_epoch = draw_epoch();
        w->have_last = false;
        w->closed.clear();
        w->pending.clear();
    }
    if (!w->open) {
        uint64_t dropped = 0;
        if (w->have_last && b.first_index > w->last_end) dropped = b.first_index - w->last_end;
        else if (loss) dropped = b.dropped_before;
        if (int32_t st = open_segment(w, b, dropped)) return st;
    }
    if (byte_count > 0 && fwrite(bytes, 1, byte_count, w->out) != byte_count)
        return set_error_fmt(RV_ERR_INVALID, "capture: writing %s failed (disk full?)", w->stem.c_str());
    w->bytes += byte_count;
    w->info.sample_count += b.sample_count;
    w->last_end = w->info.end_index();
    w->have_last = true;
    w->stats.bytes_written += byte_count;
    return rv::clear_error();
}

int32_t rv_capture_writer_set_gain(rv_capture_writer* w, int32_t has_gain, double gain_db) {
    if (w == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_set_gain: NULL");
    w->has_gain = has_gain != 0;
    w->gain_db = gain_db;
    return rv::clear_error();
}

int32_t rv_capture_writer_annotate(rv_capture_writer* w, uint64_t absolute_start, const rv_capture_annotation* a) {
    if (w == nullptr || a == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_annotate: NULL argument");
    route(w, absolute_start, *a);
    return rv::clear_error();
}

int32_t rv_capture_writer_set_clock(rv_capture_writer* w, int64_t now_ns) {
    if (w == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_set_clock: NULL");
    w->clock_ns = now_ns;
    return rv::clear_error();
}

int32_t rv_capture_writer_get_stats(const rv_capture_writer* w, rv_capture_writer_stats* out) {
    if (w == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_writer_get_stats: NULL");
    *out = w->stats;
    out->stream_epoch = w->config.stream_epoch;
    return rv::clear_error();
}

int32_t rv_capture_writer_close(rv_capture_writer* w) {
    if (w == nullptr) return rv::clear_error();
    const int32_t st = close_segment(w, "stop");
    if (w->out) fclose(w->out);
    delete w;
    return st ? st : rv::clear_error();
}

int32_t rv_capture_recover(const char* root, uint32_t counts[3]) {
    if (root == nullptr || counts == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_recover: NULL argument");
    recover(root, counts);
    return rv::clear_error();
}

// The catalog: every closed segment under root, by day and then stem (time
// order within a day). Open segments (no meta yet) and metas whose data is
// missing are skipped.
int32_t rv_capture_list(const char* root, rv_capture_segment* out, uint32_t capacity, uint32_t* count) {
    if (root == nullptr || count == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_list: NULL argument");
    if (!is_dir(root)) return set_error_fmt(RV_ERR_INVALID, "rv_capture_list: %s is not a directory", root);
    std::vector<rv_capture_segment> found;
    for (const std::string& day : entries(root)) {
        const std::string dir = std::string(root) + "/" + day;
        if (!is_dir(dir)) continue;
        for (const std::string& name : entries(dir)) {
            if (!ends_with(name, ".sigmf-meta")) continue;
            const std::string stem = name.substr(0, name.size() - 11);
            std::string meta, v;
            uint64_t data_bytes;
            if (!read_text(dir + "/" + name, meta) || !file_size(dir + "/" + stem + ".sigmf-data", data_bytes)) continue;
            rv_capture_segment s;
            memset(&s, 0, sizeof s);
            if (stem.size() >= sizeof s.stem || day.size() >= sizeof s.day) continue;
            memcpy(s.stem, stem.data(), stem.size());
            memcpy(s.day, day.data(), day.size());
            if (!json_field(meta, "core:datatype", v) || format_from_datatype(v) < 0) continue;
            s.format = format_from_datatype(v);
            bool ok = json_field(meta, "core:sample_rate", v) && parse_i64(v, s.rate);
            ok = ok && json_field(meta, "core:frequency", v) && parse_i64(v, s.center);
            ok = ok && json_field(meta, "revenant:stream_epoch", v) && parse_u64(v, s.stream_epoch);
            ok = ok && json_field(meta, "revenant:first_index", v) && parse_u64(v, s.first_index);
            ok = ok && json_field(meta, "revenant:epoch_anchor_ns", v) && parse_i64(v, s.epoch_anchor_ns);
            ok = ok && json_field(meta, "revenant:dropped_before", v) && parse_u64(v, s.dropped_before);
            if (!ok) continue;
            if (json_field(meta, "revenant:close_reason", v))
                snprintf(s.close_reason, sizeof s.close_reason, "%s", v.c_str());
            if (json_field(meta, "revenant:gain_db", v) && parse_f64(v, s.gain_db)) s.has_gain = 1;
            s.samples = data_bytes / bytes_per_sample(s.format);
            found.push_back(s);
        }
    }
    *count = (uint32_t)found.size();
    if (out)
        for (uint32_t i = 0; i < *count && i < capacity; ++i) out[i] = found[i];
    return rv::clear_error();
}

// Samples [offset, offset + count) of a listed segment, in its own format.
int32_t rv_capture_read(const char* root, const rv_capture_segment* seg, uint64_t offset, uint64_t count, void* out) {
    if (root == nullptr || seg == nullptr || (out == nullptr && count > 0))
        return set_error_fmt(RV_ERR_INVALID, "rv_capture_read: NULL argument");
    if (!known_format(seg->format)) return set_error_fmt(RV_ERR_INVALID, "rv_capture_read: format %d", seg->format);
    if (offset > seg->samples || count > seg->samples - offset)
        return set_error_fmt(RV_ERR_INVALID, "rv_capture_read: [%llu, +%llu) outside a %llu-sample segment",
                             (unsigned long long)offset, (unsigned long long)count, (unsigned long long)seg->samples);
    const std::string path = std::string(root) + "/" + field_text(seg->day, sizeof seg->day) + "/" +
                             field_text(seg->stem, sizeof seg->stem) + ".sigmf-data";
    FILE* f = fopen(path.c_str(), "rb");
    if (f == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_capture_read: cannot open %s", path.c_str());
    const uint64_t bps = bytes_per_sample(seg->format);
    const bool ok = fseeko(f, (off_t)(offset * bps), SEEK_SET) == 0 && fread(out, bps, count, f) == count;
    fclose(f);
    if (!ok) return set_error_fmt(RV_ERR_INVALID, "rv_capture_read: short read from %s", path.c_str());
    return rv::clear_error();
}

}  // extern "C"
