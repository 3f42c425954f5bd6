// Snapshots of the device-resident state and an append-only archive of them: the
// GPU counterpart of REBOUND's Simulationarchive (src/simulationarchive.c:377-411,
// 639-666).  A snapshot holds exactly what a restart needs to continue bit for bit:
// the configuration, the particle arrays as they are on the device (not
// synchronized), the WHFast coordinates with the synchronized / modified flags,
// dt_last_done, the SEI cache and the step count.  Saving never synchronizes, so
// taking snapshots does not change the trajectory.
//
// Archive file: records appended one after another, each a SnapHeader followed by
// 11 N doubles (x, y, z, vx, vy, vz, ax, ay, az, m, r per particle) and, when the
// handle has WHFast coordinates, 7 N doubles (x, y, z, vx, vy, vz, m per body).
// A reader stops at the first record that is cut short or does not carry the
// magic, so an interrupted write loses only the snapshot being written.
#include "rgpu_internal.cuh"
#include "whfast_plain.cuh"
#include <cstdio>
#include <cstring>

namespace {

constexpr char kMagic[8] = {'R', 'G', 'P', 'U', 'S', 'N', 'A', 'P'};
constexpr uint32_t kVersion = 1;

struct SnapHeader {
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    uint64_t record_bytes;     // header + payload
    uint64_t N;
    uint32_t flags;            // kSynchronized | kModified | kHasWhfast
    uint32_t config_bytes;
    double t;
    double dt_last_done;
    int64_t steps_done;
    double sei[5];
    rgpu_config cfg;
};
enum : uint32_t { kSynchronized = 1, kModified = 2, kHasWhfast = 4 };

size_t record_bytes(size_t N, bool whfast) {
    return sizeof(SnapHeader) + sizeof(double) * N * (11 + (whfast ? 7 : 0));
}

bool has_whfast(const rgpu_sim* s) { return s->wh && s->wh->jac && s->wh->cap >= s->N; }

bool header_ok(const SnapHeader& h, size_t avail) {
    return std::memcmp(h.magic, kMagic, 8) == 0 && h.version == kVersion && h.header_bytes == sizeof(SnapHeader) &&
           h.config_bytes == sizeof(rgpu_config) && h.N < ((uint64_t)1 << 31) &&
           h.record_bytes == record_bytes((size_t)h.N, (h.flags & kHasWhfast) != 0) && h.record_bytes <= avail;
}

// Walks the records of an archive file: calls f(header, offset) for each whole one.
template <class F>
int scan_file(const char* path, F&& f) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return RGPU_ERR_ARG;
    std::fseek(fp, 0, SEEK_END);
    const long long size = std::ftell(fp);
    long long off = 0;
    while (off + (long long)sizeof(SnapHeader) <= size) {
        SnapHeader h;
        std::fseek(fp, off, SEEK_SET);
        if (std::fread(&h, sizeof h, 1, fp) != 1 || !header_ok(h, (size_t)(size - off))) break;
        if (!f(h, off)) break;
        off += (long long)h.record_bytes;
    }
    std::fclose(fp);
    return RGPU_OK;
}

}  // namespace

extern "C" int rgpu_sim_snapshot_size(rgpu_sim* s, size_t* bytes) {
    if (!s || !bytes) return RGPU_ERR_ARG;
    *bytes = record_bytes(s->N, has_whfast(s));
    return RGPU_OK;
}

extern "C" int rgpu_sim_snapshot_write(rgpu_sim* s, void* buf, size_t cap, size_t* written) {
    if (!s || !buf || !written) return RGPU_ERR_ARG;
    const bool wh = has_whfast(s);
    const size_t need = record_bytes(s->N, wh);
    *written = 0;
    if (cap < need) return set_error(s, RGPU_ERR_OVERFLOW, "snapshot buffer too small");
    SnapHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.header_bytes = sizeof(SnapHeader);
    h.record_bytes = need;
    h.N = s->N;
    h.flags = (s->whfast_synchronized ? kSynchronized : 0) | (s->did_modify ? kModified : 0) | (wh ? kHasWhfast : 0);
    h.config_bytes = sizeof(rgpu_config);
    h.t = s->cfg.t;
    h.dt_last_done = s->dt_last_done;
    h.steps_done = s->steps_done;
    h.sei[0] = s->sei.lastdt; h.sei[1] = s->sei.sindt; h.sei[2] = s->sei.tandt;
    h.sei[3] = s->sei.sindtz; h.sei[4] = s->sei.tandtz;
    h.cfg = s->cfg;
    char* out = static_cast<char*>(buf);
    std::memcpy(out, &h, sizeof h);
    double* p = reinterpret_cast<double*>(out + sizeof h);
    if (s->N) RGPU_TRY(rgpu_sim_get_particles(s, p, s->N, 88));       // the device state as it is
    if (wh) {
        double* q = p + 11 * s->N;
        for (int f = 0; f < 7; f++)
            RGPU_CUDA(s, cudaMemcpyAsync(q + f * s->N, s->wh->jac + f * s->wh->cap, sizeof(double) * s->N,
                                         cudaMemcpyDeviceToHost, s->stream));
        RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    }
    *written = need;
    return RGPU_OK;
}

extern "C" int rgpu_sim_snapshot_read(rgpu_sim* s, const void* buf, size_t n) {
    if (!s || !buf) return RGPU_ERR_ARG;
    SnapHeader h;
    if (n < sizeof h) return set_error(s, RGPU_ERR_ARG, "snapshot too short");
    std::memcpy(&h, buf, sizeof h);
    if (!header_ok(h, n)) return set_error(s, RGPU_ERR_ARG, "not a snapshot of this library (magic, version or size)");
    RGPU_TRY(rgpu_sim_configure(s, &h.cfg));
    const double* p = reinterpret_cast<const double*>(static_cast<const char*>(buf) + sizeof h);
    RGPU_TRY(rgpu_sim_set_particles(s, p, (size_t)h.N, 88));
    if (h.flags & kHasWhfast) RGPU_TRY(whfast_load_coordinates(s, p + 11 * h.N));
    s->whfast_synchronized = (h.flags & kSynchronized) != 0;
    s->did_modify = (h.flags & kModified) != 0;
    s->dt_last_done = h.dt_last_done;
    s->steps_done = h.steps_done;
    s->sei.lastdt = h.sei[0]; s->sei.sindt = h.sei[1]; s->sei.tandt = h.sei[2];
    s->sei.sindtz = h.sei[3]; s->sei.tandtz = h.sei[4];
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    return RGPU_OK;
}

// Appends one snapshot of the handle to the archive file.
int archive_append(rgpu_sim* s, const char* path) {
    size_t bytes = 0;
    RGPU_TRY(rgpu_sim_snapshot_size(s, &bytes));
    std::vector<char> buf(bytes);
    size_t written = 0;
    RGPU_TRY(rgpu_sim_snapshot_write(s, buf.data(), bytes, &written));
    FILE* fp = std::fopen(path, "ab");
    if (!fp) return set_error(s, RGPU_ERR_ARG, std::string("cannot open archive ") + path);
    const bool ok = std::fwrite(buf.data(), 1, written, fp) == written;
    std::fclose(fp);
    if (!ok) return set_error(s, RGPU_ERR_ARG, std::string("short write to archive ") + path);
    return RGPU_OK;
}

// reb_simulationarchive_heartbeat (src/simulationarchive.c:377-408): a snapshot
// whenever t passes the next output time (interval) or the step count reaches the
// next output step.
int archive_heartbeat(rgpu_sim* s) {
    if (s->archive_path.empty()) return RGPU_OK;
    if (s->archive_interval != 0.) {
        const double sign = s->cfg.dt > 0. ? 1. : -1;
        if (sign * s->archive_next <= sign * s->cfg.t) {
            s->archive_next += sign * s->archive_interval;
            return archive_append(s, s->archive_path.c_str());
        }
    }
    if (s->archive_step != 0) {
        if (s->archive_next_step <= s->steps_done) {
            s->archive_next_step += s->archive_step;
            return archive_append(s, s->archive_path.c_str());
        }
    }
    return RGPU_OK;
}

extern "C" int rgpu_sim_save_to_file(rgpu_sim* s, const char* path, double interval, int64_t step, int delete_file) {
    if (!s || !path || !*path) return RGPU_ERR_ARG;
    if (interval != 0. && step != 0) return set_error(s, RGPU_ERR_ARG, "Only use one of interval or step");
    if (delete_file) std::remove(path);
    if (interval == 0. && step == 0) return archive_append(s, path);          // reb_simulation_save_to_file
    s->archive_path = path;
    if (interval != 0. && s->archive_interval != interval) {                  // :639-648
        s->archive_interval = interval;
        s->archive_next = s->cfg.t;
    }
    if (step != 0 && s->archive_step != step) {                               // :657-666
        s->archive_step = step;
        s->archive_next_step = s->steps_done;
    }
    return RGPU_OK;
}

extern "C" int rgpu_archive_scan(const char* path, double* times, int64_t* offsets, size_t cap, size_t* n) {
    if (!path || !n || (cap && (!times || !offsets))) return RGPU_ERR_ARG;
    size_t k = 0;
    const int rc = scan_file(path, [&](const SnapHeader& h, long long off) {
        if (k < cap) { times[k] = h.t; offsets[k] = off; }
        k++;
        return true;
    });
    *n = k;
    if (rc) return rc;
    return k > cap ? RGPU_ERR_OVERFLOW : RGPU_OK;
}

extern "C" int rgpu_sim_load_from_file(rgpu_sim* s, const char* path, int64_t index) {
    if (!s || !path) return RGPU_ERR_ARG;
    std::vector<long long> offs;
    std::vector<uint64_t> sizes;
    if (scan_file(path, [&](const SnapHeader& h, long long off) {
            offs.push_back(off);
            sizes.push_back(h.record_bytes);
            return true;
        }))
        return set_error(s, RGPU_ERR_ARG, std::string("cannot read archive ") + path);
    const int64_t n = (int64_t)offs.size();
    if (index < 0) index += n;
    if (index < 0 || index >= n) return set_error(s, RGPU_ERR_ARG, "snapshot index out of range");
    std::vector<char> buf(sizes[index]);
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return set_error(s, RGPU_ERR_ARG, std::string("cannot read archive ") + path);
    std::fseek(fp, offs[index], SEEK_SET);
    const bool ok = std::fread(buf.data(), 1, buf.size(), fp) == buf.size();
    std::fclose(fp);
    if (!ok) return set_error(s, RGPU_ERR_ARG, "archive changed while reading");
    return rgpu_sim_snapshot_read(s, buf.data(), buf.size());
}
