// writer.cpp -- output file sets (include/corr_writer.h).
//
// The on-disk contract of the reference's host writer (corr-rs/src/writer.rs):
// one raw complex64 file per baseline plus four sidecars per set, the set named
// by the local time of its first row, whole rows only, data before sidecars,
// resume by the shortest file, a new set per local day. The names, line formats
// and metadata keys are kept exactly because downstream readers parse them; the
// code is this library's own: POSIX file descriptors, one writer thread fed from
// a bounded queue of row buffers, errors reported through corr_last_error().
//
// Map to the reference:
//   set names                    writer.rs:88-148 (SetNames)
//   writing one row              writer.rs:796-866 (write_one)
//   resume / truncation          writer.rs:351-530 (attach), :1753-1864 (helpers)
//   opening and rolling sets     writer.rs:575-782, :1652-1659 (decide)
//   discovering sets             writer.rs:1672-1730
//   metadata.yaml                writer.rs:1867-1973
//   queue: drop or block         writer.rs:1485-1556

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <deque>
#include <filesystem>
#include <fstream>
#include <memory>
#include <mutex>
#include <optional>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "corr_writer.h"
#include "engine.h"

namespace corrgb {
namespace {

namespace fs = std::filesystem;

constexpr size_t kTextFlushBytes = 8192;   // sidecar text buffered up to this much

// Outcome of a step inside the writer: a status and its message.
struct Err {
    corr_status st = CORR_OK;
    std::string msg;
    explicit operator bool() const { return st != CORR_OK; }
};

Err io_error(const std::string &what, const std::string &path) {
    return {CORR_ERR_INTERNAL, what + " " + path + ": " + std::strerror(errno)};
}

int64_t now_ms() {
    return std::chrono::duration_cast<std::chrono::milliseconds>(
               std::chrono::system_clock::now().time_since_epoch())
        .count();
}

int64_t floor_div(int64_t a, int64_t b) { return a / b - ((a % b != 0) && ((a < 0) != (b < 0))); }

// strftime of the local time at `ms` (writer's config.rs stamp_at).
std::string local_stamp(int64_t ms, const char *fmt) {
    const time_t secs = static_cast<time_t>(floor_div(ms, 1000));
    struct tm tm;
    std::memset(&tm, 0, sizeof tm);
    if (localtime_r(&secs, &tm) == nullptr) return "unknown_time";
    char buf[128];
    const size_t n = std::strftime(buf, sizeof buf, fmt, &tm);
    if (n == 0) return "unknown_time";
    return std::string(buf, n);
}

std::string local_day(int64_t ms) { return local_stamp(ms, "%Y%m%d"); }

long local_utc_offset_s(int64_t ms) {
    const time_t secs = static_cast<time_t>(floor_div(ms, 1000));
    struct tm tm;
    std::memset(&tm, 0, sizeof tm);
    if (localtime_r(&secs, &tm) == nullptr) return 0;
    return tm.tm_gmtoff;
}

// One row's wall clock as a line of time.txt: local date and time, milliseconds.
std::string text_time(int64_t ms) {
    char frac[8];
    std::snprintf(frac, sizeof frac, ".%03lld",
                  static_cast<long long>(ms - floor_div(ms, 1000) * 1000));
    return local_stamp(ms, "%Y-%m-%d %H:%M:%S") + frac;
}

// A double as the reference's metadata prints it: the shortest decimal that
// reads back to the same value, never in exponent form.
std::string fmt_f64(double v) {
    char buf[400];
    auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::fixed);
    return std::string(buf, r.ptr);
}

struct Names {
    std::string prefix, stamp;
    std::string tag() const { return prefix + stamp; }
    std::string baseline(const std::string &j, const std::string &k) const {
        return prefix + j + k + "-" + stamp + ".bin";
    }
    std::string time_txt() const { return tag() + "-time.txt"; }
    std::string time_bin() const { return tag() + "-time.bin"; }
    std::string blocks() const { return tag() + "-blocks.csv"; }
    std::string metadata() const { return tag() + "-metadata.yaml"; }
};

uint64_t file_len(const std::string &p) {
    struct stat st;
    return ::stat(p.c_str(), &st) == 0 ? static_cast<uint64_t>(st.st_size) : 0;
}

bool file_exists(const std::string &p) {
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

bool read_file(const std::string &p, std::string *out) {
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    *out = ss.str();
    return true;
}

std::vector<std::string> lines_of(const std::string &s) {
    std::vector<std::string> out;
    size_t a = 0;
    while (a < s.size()) {
        size_t b = s.find('\n', a);
        if (b == std::string::npos) b = s.size();
        out.push_back(s.substr(a, b - a));
        a = b + 1;
    }
    return out;
}

std::string trim(const std::string &s) {
    const size_t a = s.find_first_not_of(" \t\r");
    if (a == std::string::npos) return "";
    return s.substr(a, s.find_last_not_of(" \t\r") - a + 1);
}

bool is_data_line(const std::string &l) { return !l.empty() && l[0] != '#'; }

std::optional<std::string> read_metadata_field(const std::string &path, const std::string &key) {
    std::string s;
    if (!read_file(path, &s)) return std::nullopt;
    const std::string want = key + ":";
    for (const std::string &l : lines_of(s))
        if (l.compare(0, want.size(), want) == 0) return trim(l.substr(want.size()));
    return std::nullopt;
}

uint64_t count_csv_rows(const std::string &p) {
    std::string s;
    if (!read_file(p, &s)) return 0;
    uint64_t n = 0;
    for (const std::string &l : lines_of(s)) n += is_data_line(l);
    return n;
}

Err write_whole(int fd, const void *data, size_t n, const std::string &path) {
    const char *p = static_cast<const char *>(data);
    while (n > 0) {
        const ssize_t w = ::write(fd, p, n);
        if (w < 0) {
            if (errno == EINTR) continue;
            return io_error("writing", path);
        }
        p += w;
        n -= static_cast<size_t>(w);
    }
    return {};
}

Err write_text_file(const std::string &p, const std::string &s) {
    const int fd = ::open(p.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return io_error("creating", p);
    Err e = write_whole(fd, s.data(), s.size(), p);
    ::close(fd);
    return e;
}

Err truncate_to(const std::string &p, uint64_t len) {
    if (file_exists(p) && file_len(p) == len) return {};
    const int fd = ::open(p.c_str(), O_WRONLY | O_CREAT, 0644);
    if (fd < 0) return io_error("opening", p);
    const int r = ::ftruncate(fd, static_cast<off_t>(len));
    Err e = r != 0 ? io_error("truncating", p) : Err{};
    ::close(fd);
    return e;
}

// Keep the comment lines and the first `keep` data lines of a csv.
Err truncate_csv(const std::string &p, uint64_t keep) {
    std::string s;
    if (!read_file(p, &s) || s.empty()) return {};
    std::string head, data;
    uint64_t n = 0, total = 0;
    for (const std::string &l : lines_of(s)) {
        if (!l.empty() && l[0] == '#') {
            head += l + "\n";
        } else if (is_data_line(l)) {
            ++total;
            if (n < keep) {
                data += l + "\n";
                ++n;
            }
        }
    }
    if (total == keep) return {};
    return write_text_file(p, head + data);
}

// First frame of the row after the last one in blocks.csv (writer.rs:1841-1864).
std::optional<uint64_t> next_frame_after(const std::string &blocks, uint32_t n_cum) {
    std::string s;
    if (!read_file(blocks, &s)) return std::nullopt;
    std::string last;
    for (const std::string &l : lines_of(s))
        if (is_data_line(l)) last = l;
    if (last.empty()) return std::nullopt;
    std::vector<std::string> col;
    std::stringstream ss(last);
    std::string c;
    while (std::getline(ss, c, ',')) col.push_back(c);
    uint64_t first = 0;
    if (col.size() > 2) first = std::strtoull(col[2].c_str(), nullptr, 10);
    return first + n_cum;
}

enum class SetKind { Start, Rollover, Resume, SecondSet };
const char *kind_name(SetKind k) {
    switch (k) {
    case SetKind::Start: return "start";
    case SetKind::Rollover: return "rollover";
    case SetKind::Resume: return "resume";
    case SetKind::SecondSet: return "second_set";
    }
    return "start";
}

struct FoundSet {
    std::string tag;
    Names names;
    std::string day;
    uint64_t rows = 0;
};

struct Job {
    std::vector<char> row;
    int64_t ms = 0;
    uint64_t row_index = 0, first_frame_id = 0;
    std::vector<uint64_t> valid;
};

class Writer {
public:
    // ---- configuration (immutable after open) ----
    std::string dir, file_prefix, prefix_format, config_version, config_hash;
    std::vector<std::string> st_name, st_ip, st_board;
    std::vector<int32_t> st_port;
    std::vector<bool> st_has_net;
    int n_station = 0, n_freq = 0, n_baseline = 0;
    uint32_t n_cum = 0, frames_per_slot = 0, rows_per_fetch = 0, fsync_every = 1;
    uint64_t sample_rate_hz = 0;
    int32_t data_shift_count = 0;
    bool daily = true;
    int queue_full = CORRW_QUEUE_DROP;
    uint32_t queue_rows = 0;
    size_t per_baseline_row = 0, row_bytes = 0;
    std::vector<std::pair<int, int>> pairs;

    // ---- set state (the writer thread's, or the caller's when synchronous) ----
    bool have_set = false;
    Names names;
    std::string set_day;
    SetKind set_kind = SetKind::Start;
    uint64_t rows_in_set = 0, rows_total = 0;
    std::atomic<uint64_t> rows_done{0};      // rows_total, readable from any thread
    std::atomic<uint32_t> sets_opened{0};
    bool backward_warned = false;
    std::vector<int> fd_base;
    int fd_ms_bin = -1, fd_ms_txt = -1, fd_blocks = -1;
    std::string txt_buf, blocks_buf;

    // ---- queue (guarded by mu) ----
    std::mutex mu;
    std::condition_variable cv_work, cv_idle;
    std::deque<Job> queue;
    std::vector<std::vector<char>> pool;
    bool busy = false, stopping = false;
    Err error;
    uint64_t dropped = 0, max_queued = 0;
    std::string live_tag;
    std::thread thread;

    std::string path(const std::string &name) const { return (fs::path(dir) / name).string(); }
    std::string baseline_path(const Names &n, int b) const {
        return path(n.baseline(st_name[pairs[b].first], st_name[pairs[b].second]));
    }

    void close_files() {
        for (int fd : fd_base)
            if (fd >= 0) ::close(fd);
        fd_base.clear();
        for (int *fd : {&fd_ms_bin, &fd_ms_txt, &fd_blocks}) {
            if (*fd >= 0) ::close(*fd);
            *fd = -1;
        }
    }

    Err flush_text() {
        if (!txt_buf.empty()) {
            if (Err e = write_whole(fd_ms_txt, txt_buf.data(), txt_buf.size(),
                                    path(names.time_txt())))
                return e;
            txt_buf.clear();
        }
        if (!blocks_buf.empty()) {
            if (Err e = write_whole(fd_blocks, blocks_buf.data(), blocks_buf.size(),
                                    path(names.blocks())))
                return e;
            blocks_buf.clear();
        }
        return {};
    }

    // Flush and fsync every file of the open set, then let go of it.
    Err finish_set() {
        if (!have_set) return {};
        Err e = flush_text();
        for (size_t b = 0; b < fd_base.size() && !e; ++b)
            if (::fsync(fd_base[b]) != 0) e = io_error("fsync", baseline_path(names, int(b)));
        if (!e && ::fsync(fd_ms_bin) != 0) e = io_error("fsync", path(names.time_bin()));
        if (!e && ::fsync(fd_ms_txt) != 0) e = io_error("fsync", path(names.time_txt()));
        if (!e && ::fsync(fd_blocks) != 0) e = io_error("fsync", path(names.blocks()));
        return e;
    }

    Err write_metadata(const Names &n, const std::string &day, SetKind kind,
                       const std::string *continuation, std::optional<std::pair<uint64_t, uint64_t>> first,
                       uint64_t rows_at_open) const {
        const double frame_rate = double(sample_rate_hz) / double(2 * uint64_t(n_freq));
        std::ostringstream s;
        s << "# Written once, when this file set is created. A resumed run checks\n"
          << "# the config_hash rather than rewriting geometry that the existing\n"
          << "# rows were produced with.\n"
          << "config_version: " << config_version << "\n"
          << "config_hash: " << config_hash << "\n"
          << "format: raw-complex64\n"
          << "byte_order: little_endian\n"
          << "component: {real: float32, imag: float32}\n"
          << "baseline_layout: baseline_major\n"
          << "n_freq: " << n_freq << "\n"
          << "n_cum: " << n_cum << "\n"
          << "n_station: " << n_station << "\n"
          << "n_baseline: " << n_baseline << "\n"
          << "sample_rate_hz: " << sample_rate_hz << "\n"
          << "bin_width_hz: " << fmt_f64(frame_rate) << "\n"
          << "frame_rate_hz: " << fmt_f64(frame_rate) << "\n"
          << "row_period_s: " << fmt_f64(double(n_cum) / frame_rate) << "\n"
          << "fft: {type: R2C, length: " << 2 * n_freq
          << ", window: rectangular, nyquist: dropped}\n"
          << "fft_normalisation: none\n"
          << "row_normalisation: divide_by_n_cum\n"
          << "missing_frames: zero_filled\n"
          << "fftshift: false\n"
          << "bin0: DC\n"
          << "data_shift_count: " << data_shift_count << "\n"
          << "frames_per_slot: " << frames_per_slot << "\n"
          << "rows_per_fetch: " << rows_per_fetch << "\n"
          << "baseline_row_bytes: " << per_baseline_row << "\n"
          << "# --- the file set this metadata belongs to ---\n"
          << "set_prefix: " << n.tag() << "\n"
          << "rows_ms_txt_format: \"local YYYY-mm-DD HH:MM:SS.mmm\"\n"
          << "file_prefix: " << n.prefix << "\n"
          << "stamp: " << n.stamp << "\n"
          << "set_day: " << day << "\n"
          << "set_kind: " << kind_name(kind) << "\n";
        if (continuation) s << "set_continuation_of: " << *continuation << "\n";
        s << "first_row_index: " << (first ? first->first : 0) << "\n"
          << "first_frame_id: " << (first ? first->second : 0) << "\n"
          << "rows_at_open: " << rows_at_open << "\n";
        const char *tz = std::getenv("TZ");
        s << "local_timezone: " << (tz ? tz : "") << "\n"
          << "local_utc_offset_s: " << local_utc_offset_s(now_ms()) << "\n"
          << "stations:\n";
        for (int i = 0; i < n_station; ++i) {
            s << "  - {index: " << i << ", name: " << st_name[i];
            if (st_has_net[i])
                s << ", group_ip: " << st_ip[i] << ", dest_port: " << st_port[i]
                  << ", board: " << st_board[i];
            s << "}\n";
        }
        s << "baselines:\n";
        for (int b = 0; b < n_baseline; ++b)
            s << "  - {index: " << b << ", j: " << pairs[b].first << ", k: " << pairs[b].second
              << ", file: " << n.baseline(st_name[pairs[b].first], st_name[pairs[b].second])
              << "}\n";
        return write_text_file(path(n.metadata()), s.str());
    }

    Err open_append(const std::string &p, uint64_t pos, bool at_end, int *fd) {
        *fd = ::open(p.c_str(), O_WRONLY | O_CREAT, 0644);
        if (*fd < 0) return io_error("opening", p);
        const off_t r = at_end ? ::lseek(*fd, 0, SEEK_END) : ::lseek(*fd, off_t(pos), SEEK_SET);
        if (r < 0) return io_error("seeking", p);
        return {};
    }

    // Attach to the set `n` (new or existing): truncate to whole rows, reopen for
    // appending, write or check metadata (writer.rs:351-530).
    Err attach(const Names &n, const FoundSet *found, corrw_resume *resume) {
        uint64_t complete = UINT64_MAX;
        std::vector<uint64_t> sizes(n_baseline);
        for (int b = 0; b < n_baseline; ++b) {
            sizes[b] = file_len(baseline_path(n, b));
            complete = std::min<uint64_t>(complete, sizes[b] / per_baseline_row);
        }
        if (complete == UINT64_MAX) complete = 0;
        const uint64_t ms_rows = file_len(path(n.time_bin())) / 8;
        const uint64_t blocks_rows = count_csv_rows(path(n.blocks())) / uint64_t(n_station);
        const uint64_t rows = std::min({complete, ms_rows, blocks_rows});
        const uint64_t truncated = complete > rows ? complete - rows : 0;

        for (int b = 0; b < n_baseline; ++b)
            if (sizes[b] != rows * per_baseline_row || !file_exists(baseline_path(n, b)))
                if (Err e = truncate_to(baseline_path(n, b), rows * per_baseline_row)) return e;
        if (Err e = truncate_to(path(n.time_bin()), rows * 8)) return e;
        if (Err e = truncate_csv(path(n.blocks()), rows * uint64_t(n_station))) return e;
        // time.txt is derived from time.bin, so it is rebuilt rather than truncated
        {
            std::string bin, txt;
            read_file(path(n.time_bin()), &bin);
            for (uint64_t r = 0; r < rows && (r + 1) * 8 <= bin.size(); ++r) {
                uint64_t u = 0;
                for (int i = 7; i >= 0; --i) u = (u << 8) | uint8_t(bin[r * 8 + i]);
                txt += text_time(static_cast<int64_t>(u)) + "\n";
            }
            if (Err e = write_text_file(path(n.time_txt()), txt)) return e;
        }
        const std::optional<uint64_t> next = next_frame_after(path(n.blocks()), n_cum);

        fd_base.assign(n_baseline, -1);
        for (int b = 0; b < n_baseline; ++b)
            if (Err e = open_append(baseline_path(n, b), rows * per_baseline_row, false, &fd_base[b]))
                return e;
        if (Err e = open_append(path(n.time_bin()), rows * 8, false, &fd_ms_bin)) return e;
        if (Err e = open_append(path(n.time_txt()), 0, true, &fd_ms_txt)) return e;
        if (Err e = open_append(path(n.blocks()), 0, true, &fd_blocks)) return e;

        const std::string meta = path(n.metadata());
        const bool created_now = rows == 0 || !file_exists(meta);
        const std::string day = found ? found->day : local_day(now_ms());
        if (created_now) {
            if (Err e = write_metadata(n, day, SetKind::Start, nullptr, std::nullopt, rows)) return e;
        } else {
            const std::string have = read_metadata_field(meta, "config_hash").value_or("");
            if (have != config_hash)
                return {CORR_ERR_STATE, meta + " was written with config_hash " + have +
                                            " but this writer has " + config_hash +
                                            "; resuming would misinterpret every existing row"};
        }
        names = n;
        have_set = true;
        set_day = day;
        set_kind = created_now ? SetKind::Start : SetKind::Resume;
        rows_in_set = rows;
        rows_total = rows;
        rows_done = rows;
        ++sets_opened;
        if (resume) {
            resume->rows_written = rows;
            resume->truncated_rows = truncated;
            resume->has_next_frame_id = next.has_value();
            resume->next_frame_id = next.value_or(0);
        }
        return {};
    }

    Err try_create_set(const Names &n, const std::string &day, SetKind kind,
                       const std::string *continuation, const Job &job) {
        const std::string probe = baseline_path(n, 0);
        if (file_exists(probe) && file_len(probe) > 0)
            return {CORR_ERR_STATE, probe + " already holds " + std::to_string(file_len(probe)) +
                                        " bytes: the set tag " + n.tag() + " is in use"};
        std::vector<int> fds(n_baseline, -1);
        auto create = [&](const std::string &p, int *fd) -> Err {
            *fd = ::open(p.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
            return *fd < 0 ? io_error("creating", p) : Err{};
        };
        Err e;
        for (int b = 0; b < n_baseline && !e; ++b) e = create(baseline_path(n, b), &fds[b]);
        int fbin = -1, ftxt = -1, fblk = -1;
        if (!e) e = create(path(n.time_bin()), &fbin);
        if (!e) e = create(path(n.time_txt()), &ftxt);
        if (!e) e = create(path(n.blocks()), &fblk);
        if (!e)
            e = write_metadata(n, day, kind, continuation,
                               std::make_pair(job.row_index, job.first_frame_id), 0);
        if (e) {
            for (int fd : fds)
                if (fd >= 0) ::close(fd);
            for (int fd : {fbin, ftxt, fblk})
                if (fd >= 0) ::close(fd);
            return e;
        }
        fd_base = std::move(fds);
        fd_ms_bin = fbin;
        fd_ms_txt = ftxt;
        fd_blocks = fblk;
        names = n;
        have_set = true;
        set_day = day;
        set_kind = kind;
        rows_in_set = 0;
        ++sets_opened;
        return {};
    }

    Err create_set(const std::string &day, const Job &job, SetKind kind,
                   const std::string *continuation) {
        const Names n{file_prefix, local_stamp(job.ms, prefix_format.c_str())};
        Err last;
        for (int attempt = 1; attempt <= 3; ++attempt) {
            last = try_create_set(n, day, kind, continuation, job);
            if (!last) return {};
            if (last.st == CORR_ERR_STATE) break;     // a tag in use does not heal
            if (attempt < 3) std::this_thread::sleep_for(std::chrono::milliseconds(100));
        }
        return {last.st, "opening file set " + n.tag() + " for local day " + day + ": " + last.msg};
    }

    // The set a row belongs to: open, keep or roll by its local day.
    Err ensure_set_for(const Job &job) {
        if (!daily) {
            if (!have_set) return {CORR_ERR_INTERNAL, "no output set is open"};
            return {};
        }
        const std::string day = local_day(job.ms);
        if (!have_set) return create_set(day, job, set_kind, nullptr);
        if (day == set_day) return {};
        if (day > set_day) {
            const uint64_t rows = rows_in_set;
            const std::string from_day = set_day, from = names.tag();
            if (Err e = finish_set()) return e;
            close_files();
            have_set = false;
            if (Err e = create_set(day, job, SetKind::Rollover, &from)) return e;
            std::fprintf(stderr,
                         "writer: local day changed %s -> %s: closed set %s (%llu rows) and "
                         "opened %s\n",
                         from_day.c_str(), day.c_str(), from.c_str(),
                         static_cast<unsigned long long>(rows), names.tag().c_str());
            return {};
        }
        if (!backward_warned) {
            backward_warned = true;
            std::fprintf(stderr,
                         "writer: the local day went backwards (%s -> %s); keeping set %s\n",
                         set_day.c_str(), day.c_str(), names.tag().c_str());
        }
        return {};
    }

    // One row: spectra first (one write per baseline), then the sidecars.
    Err write_one(const Job &job, const char *row) {
        if (Err e = ensure_set_for(job)) return e;
        {
            std::lock_guard<std::mutex> lk(mu);
            live_tag = names.tag();
        }
        const bool sync_now = rows_total % fsync_every == 0;
        for (int b = 0; b < n_baseline; ++b)
            if (Err e = write_whole(fd_base[b], row + size_t(b) * per_baseline_row,
                                    per_baseline_row, baseline_path(names, b)))
                return e;
        if (sync_now)
            for (int b = 0; b < n_baseline; ++b)
                if (::fdatasync(fd_base[b]) != 0) return io_error("fdatasync", baseline_path(names, b));
        unsigned char le[8];
        const uint64_t u = static_cast<uint64_t>(job.ms);
        for (int i = 0; i < 8; ++i) le[i] = static_cast<unsigned char>(u >> (8 * i));
        if (Err e = write_whole(fd_ms_bin, le, 8, path(names.time_bin()))) return e;
        txt_buf += text_time(job.ms) + "\n";
        for (int s = 0; s < n_station; ++s) {
            const uint64_t valid = job.valid[s];
            blocks_buf += std::to_string(job.row_index) + "," + std::to_string(s) + "," +
                          std::to_string(job.first_frame_id) + "," + std::to_string(n_cum) + "," +
                          std::to_string(valid) + "," + std::to_string(uint64_t(n_cum) - valid) +
                          "\n";
        }
        if (sync_now || txt_buf.size() > kTextFlushBytes || blocks_buf.size() > kTextFlushBytes)
            if (Err e = flush_text()) return e;
        ++rows_total;
        ++rows_in_set;
        rows_done = rows_total;
        return {};
    }

    void run() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv_work.wait(lk, [&] { return stopping || !queue.empty(); });
            if (queue.empty()) break;               // stopping, nothing left
            Job job = std::move(queue.front());
            queue.pop_front();
            busy = true;
            const bool failed = bool(error);
            lk.unlock();
            Err e = failed ? Err{} : write_one(job, job.row.data());
            lk.lock();
            if (e && !error) error = e;
            pool.push_back(std::move(job.row));
            busy = false;
            cv_idle.notify_all();
        }
    }
};

// Every set already in the directory, by its blocks.csv and metadata (writer.rs:1672-1730).
std::vector<FoundSet> discover_sets(const Writer &w) {
    std::vector<FoundSet> out;
    std::error_code ec;
    for (const auto &ent : fs::directory_iterator(w.dir, ec)) {
        const std::string name = ent.path().filename().string();
        const std::string suffix = "-blocks.csv";
        if (name.size() <= suffix.size() ||
            name.compare(name.size() - suffix.size(), suffix.size(), suffix) != 0)
            continue;
        const std::string tag = name.substr(0, name.size() - suffix.size());
        const std::string meta = w.path(tag + "-metadata.yaml");
        const auto stamp = read_metadata_field(meta, "stamp");
        if (!stamp) continue;
        FoundSet f;
        f.tag = tag;
        f.names = Names{read_metadata_field(meta, "file_prefix").value_or(""), *stamp};
        f.day = read_metadata_field(meta, "set_day").value_or("");
        out.push_back(f);
    }
    std::sort(out.begin(), out.end(),
              [](const FoundSet &a, const FoundSet &b) { return a.tag < b.tag; });
    return out;
}

corr_status report(const Err &e) { return e ? fail(e.st, e.msg) : CORR_OK; }

}  // namespace
}  // namespace corrgb

using namespace corrgb;

extern "C" corr_status corrw_open(const corrw_params *p, void **out_writer, corrw_resume *resume) {
    if (p == nullptr || out_writer == nullptr) return fail(CORR_ERR_ARG, "NULL argument");
    *out_writer = nullptr;
    if (p->struct_size != sizeof(corrw_params))
        return failf(CORR_ERR_ABI, "corrw_params.struct_size=%u, expected %zu", p->struct_size,
                     sizeof(corrw_params));
    if (resume != nullptr && resume->struct_size != sizeof(corrw_resume))
        return failf(CORR_ERR_ABI, "corrw_resume.struct_size=%u, expected %zu",
                     resume->struct_size, sizeof(corrw_resume));
    if (p->n_station < 1 || p->n_station > 64 || p->n_freq < 1 || p->n_cum < 1)
        return fail(CORR_ERR_ARG, "n_station must be 1..64, n_freq and n_cum >= 1");
    if (p->dir == nullptr || p->stations == nullptr || p->config_hash == nullptr)
        return fail(CORR_ERR_ARG, "dir, stations and config_hash are required");
    if (p->set_policy < CORRW_SET_AUTO || p->set_policy > CORRW_SET_EXPLICIT ||
        (p->set_policy == CORRW_SET_EXPLICIT && p->set_tag == nullptr))
        return fail(CORR_ERR_ARG, "set_policy: AUTO, NEW, or EXPLICIT with set_tag");
    const char *fmt = p->file_prefix_format ? p->file_prefix_format : "%Y%m%d-%H%M%S";
    if (std::strchr(fmt, '%') == nullptr || std::strchr(fmt, '/') != nullptr)
        return fail(CORR_ERR_ARG, "file_prefix_format needs a strftime directive and no '/'");

    auto w = std::make_unique<Writer>();
    w->dir = p->dir;
    w->file_prefix = p->file_prefix ? p->file_prefix : "";
    w->prefix_format = fmt;
    w->config_version = p->config_version ? p->config_version : "";
    w->config_hash = p->config_hash;
    w->n_station = p->n_station;
    w->n_freq = p->n_freq;
    w->n_cum = p->n_cum;
    w->frames_per_slot = p->frames_per_slot;
    w->rows_per_fetch = p->rows_per_fetch;
    w->sample_rate_hz = p->sample_rate_hz;
    w->data_shift_count = p->data_shift_count;
    w->daily = p->daily_files != 0;
    w->queue_full = p->queue_full;
    w->queue_rows = p->queue_rows;
    w->fsync_every = std::max<uint32_t>(1, p->fsync_every_rows);
    for (int i = 0; i < p->n_station; ++i) {
        const corrw_station &s = p->stations[i];
        if (s.name == nullptr || s.name[0] == '\0' || std::strchr(s.name, '/') != nullptr)
            return failf(CORR_ERR_ARG, "station %d: a name without '/' is required", i);
        w->st_name.push_back(s.name);
        w->st_has_net.push_back(s.group_ip != nullptr);
        w->st_ip.push_back(s.group_ip ? s.group_ip : "");
        w->st_port.push_back(s.dest_port);
        w->st_board.push_back(s.board ? s.board : "");
    }
    for (int j = 0; j < p->n_station; ++j)
        for (int k = j; k < p->n_station; ++k) w->pairs.emplace_back(j, k);
    w->n_baseline = static_cast<int>(w->pairs.size());
    w->per_baseline_row = size_t(p->n_freq) * 8;
    w->row_bytes = w->per_baseline_row * size_t(w->n_baseline);

    std::error_code ec;
    fs::create_directories(w->dir, ec);
    if (ec) return failf(CORR_ERR_INTERNAL, "creating %s: %s", w->dir.c_str(), ec.message().c_str());

    corrw_resume r{};
    if (!w->daily) {
        // one set per open, named by the time of opening
        const Names n{w->file_prefix, local_stamp(now_ms(), fmt)};
        if (Err e = w->attach(n, nullptr, &r)) return report(e);
    } else {
        const std::string today = local_day(now_ms());
        const std::vector<FoundSet> found = discover_sets(*w);
        const FoundSet *chosen = nullptr;
        if (p->set_policy == CORRW_SET_EXPLICIT) {
            for (const FoundSet &f : found)
                if (f.tag == p->set_tag) chosen = &f;
            if (chosen == nullptr) {
                std::string have;
                for (const FoundSet &f : found) have += (have.empty() ? "" : ", ") + f.tag;
                return failf(CORR_ERR_STATE, "no file set %s in %s (sets: %s)", p->set_tag,
                             w->dir.c_str(), have.c_str());
            }
        } else if (p->set_policy == CORRW_SET_AUTO) {
            for (const FoundSet &f : found)
                if (f.day == today && (chosen == nullptr || f.tag > chosen->tag)) chosen = &f;
        }
        if (chosen != nullptr) {
            if (Err e = w->attach(chosen->names, chosen, &r)) return report(e);
        } else {
            bool second = false;
            for (const FoundSet &f : found) second |= f.day == today;
            w->set_kind = second ? SetKind::SecondSet : SetKind::Start;
        }
    }
    w->live_tag = w->have_set ? w->names.tag() : "";
    if (resume != nullptr) {
        r.struct_size = sizeof(corrw_resume);
        *resume = r;
    }
    if (w->queue_rows > 0) {
        Writer *raw = w.get();
        w->thread = std::thread([raw] { raw->run(); });
    }
    *out_writer = w.release();
    return CORR_OK;
}

extern "C" corr_status corrw_write_row(void *handle, const void *row, size_t row_bytes,
                                       int64_t row_ms, uint64_t row_index,
                                       uint64_t first_frame_id, const uint64_t *valid_frames) {
    Writer *w = static_cast<Writer *>(handle);
    if (w == nullptr || row == nullptr || valid_frames == nullptr)
        return fail(CORR_ERR_ARG, "NULL argument");
    if (row_bytes != w->row_bytes)
        return failf(CORR_ERR_ARG, "write_row got %zu bytes but one row is %zu", row_bytes,
                     w->row_bytes);
    for (int s = 0; s < w->n_station; ++s)
        if (valid_frames[s] > w->n_cum)
            return failf(CORR_ERR_ARG, "station %d: %llu valid frames of n_cum=%u", s,
                         static_cast<unsigned long long>(valid_frames[s]), w->n_cum);
    Job job;
    job.ms = row_ms;
    job.row_index = row_index;
    job.first_frame_id = first_frame_id;
    job.valid.assign(valid_frames, valid_frames + w->n_station);
    if (w->queue_rows == 0) {
        if (w->error) return report(w->error);
        w->error = w->write_one(job, static_cast<const char *>(row));
        w->live_tag = w->have_set ? w->names.tag() : "";
        return report(w->error);
    }
    std::unique_lock<std::mutex> lk(w->mu);
    if (w->error) return report(w->error);
    const auto pending = [&] { return w->queue.size() + (w->busy ? 1 : 0); };
    if (w->queue.size() >= w->queue_rows) {
        if (w->queue_full == CORRW_QUEUE_DROP) {
            ++w->dropped;
            return CORR_OK;
        }
        w->cv_idle.wait(lk, [&] { return w->queue.size() < w->queue_rows || bool(w->error); });
        if (w->error) return report(w->error);
    }
    if (!w->pool.empty()) {
        job.row = std::move(w->pool.back());
        w->pool.pop_back();
    }
    job.row.resize(row_bytes);
    std::memcpy(job.row.data(), row, row_bytes);
    w->queue.push_back(std::move(job));
    w->max_queued = std::max<uint64_t>(w->max_queued, pending());
    w->cv_work.notify_one();
    return CORR_OK;
}

extern "C" corr_status corrw_sync(void *handle) {
    Writer *w = static_cast<Writer *>(handle);
    if (w == nullptr) return fail(CORR_ERR_ARG, "NULL writer");
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv_idle.wait(lk, [&] { return w->queue.empty() && !w->busy; });
    if (w->error) return report(w->error);
    if (w->have_set) w->error = w->flush_text();
    return report(w->error);
}

extern "C" corr_status corrw_stats_get(void *handle, corrw_stats *out) {
    Writer *w = static_cast<Writer *>(handle);
    if (w == nullptr || out == nullptr) return fail(CORR_ERR_ARG, "NULL argument");
    if (out->struct_size != sizeof(corrw_stats))
        return failf(CORR_ERR_ABI, "corrw_stats.struct_size=%u, expected %zu", out->struct_size,
                     sizeof(corrw_stats));
    std::lock_guard<std::mutex> lk(w->mu);
    out->sets_opened = w->sets_opened;
    out->rows_written = w->rows_done;
    out->rows_dropped = w->dropped;
    out->max_queued = w->max_queued;
    std::snprintf(out->set_tag, sizeof out->set_tag, "%s", w->live_tag.c_str());
    return CORR_OK;
}

extern "C" corr_status corrw_close(void *handle) {
    Writer *w = static_cast<Writer *>(handle);
    if (w == nullptr) return fail(CORR_ERR_ARG, "NULL writer");
    if (w->thread.joinable()) {
        {
            std::lock_guard<std::mutex> lk(w->mu);
            w->stopping = true;
        }
        w->cv_work.notify_all();
        w->thread.join();
    }
    Err e = w->error;
    if (!e) e = w->finish_set();
    w->close_files();
    delete w;
    return report(e);
}
