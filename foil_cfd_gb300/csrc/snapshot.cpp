// Warm-start snapshots (include/foilcfd_snapshot.h): cache keys and flag
// hashes, the device-resident exact snapshot of every active level, the host
// macroscopic snapshot with its FCS1 file format, and the LRU disk cache.
// Behaviour follows src/sim/snapshot.cpp of the reference; the FCS1 byte
// layout and the key hash are kept identical so files and cache names
// interoperate.
#include "../../include/foilcfd_snapshot.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <filesystem>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "snapshot_internal.h"

namespace fs = std::filesystem;
using namespace fcfd;

namespace {

constexpr std::uint64_t kFnvBasis = 14695981039346656037ull;
constexpr std::uint64_t kFnvMul = 1099511628211ull;
constexpr std::uint32_t kFcsMagic = 0x31534346u;   // bytes 'F' 'C' 'S' '1'
constexpr std::uint32_t kFcsFormat = 1;
constexpr std::uint32_t kPayloadRawF32 = 0;
constexpr std::uint32_t kMaxIdBytes = 4096;

std::uint64_t fnv(const void* p, size_t n, std::uint64_t h = kFnvBasis) {
    const auto* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * kFnvMul;
    return h;
}

void say(char* err, size_t len, const std::string& m) {
    if (err && len) std::snprintf(err, len, "%s", m.c_str());
}

/// Owned copy of a key (the C struct only borrows its id string).
struct Key {
    std::string id;
    int bucket = 0;
    float uLat = 0.0f;
    fcfd_dims dims{0, 0, 0};
    int version = FCFD_SOLVER_VERSION;

    static Key of(const fcfd_snapshot_key* k) {
        Key r;
        if (!k) return r;
        r.id = k->geometry_id ? k->geometry_id : "";
        r.bucket = k->aoa_bucket;
        r.uLat = k->u_lat;
        r.dims = k->dims;
        r.version = k->solver_version;
        return r;
    }
    void out(fcfd_snapshot_key* k) const {
        k->geometry_id = id.c_str();
        k->aoa_bucket = bucket;
        k->u_lat = uLat;
        k->dims = dims;
        k->solver_version = version;
    }
    std::uint64_t hash() const {
        std::uint64_t h = fnv(id.data(), id.size());
        for (const void* f : {static_cast<const void*>(&bucket), static_cast<const void*>(&uLat),
                              static_cast<const void*>(&dims.nx), static_cast<const void*>(&dims.ny),
                              static_cast<const void*>(&dims.nz), static_cast<const void*>(&version)})
            h = fnv(f, 4, h);
        return h;
    }
    std::string fileName() const {
        char b[32];
        std::snprintf(b, sizeof b, "%016llx.fcs", static_cast<unsigned long long>(hash()));
        return b;
    }
};

} // namespace

// ---- keys and hashes -----------------------------------------------------------

std::uint64_t fcfd::fnv1a64(const void* p, size_t n) { return fnv(p, n); }

extern "C" int fcfd_aoa_bucket(float aoa_deg) { return static_cast<int>(std::lround(aoa_deg * 2.0f)); }

extern "C" uint64_t fcfd_snapshot_key_hash(const fcfd_snapshot_key* key) { return Key::of(key).hash(); }

extern "C" int fcfd_snapshot_key_string(const fcfd_snapshot_key* key, char* buf, size_t len) {
    if (!key || !buf || !len) return -1;
    const Key k = Key::of(key);
    const int n = std::snprintf(buf, len, "%s_a%.1f_u%.4f_%dx%dx%d_v%d", k.id.c_str(),
                                static_cast<double>(static_cast<float>(k.bucket) * 0.5f),
                                static_cast<double>(k.uLat), k.dims.nx, k.dims.ny, k.dims.nz, k.version);
    for (size_t i = 0; i < len && buf[i]; ++i)
        if (buf[i] == ':' || buf[i] == '\\' || buf[i] == '/') buf[i] = '-';
    return n < 0 ? -1 : std::min(n, static_cast<int>(len) - 1);
}

extern "C" uint64_t fcfd_hash_flags(const uint8_t* flags, size_t n) { return flags ? fnv(flags, n) : kFnvBasis; }

// ---- VRAM snapshot ---------------------------------------------------------------

struct fcfd_vram_snapshot {
    Key key;
    std::uint64_t flagsHash = 0;
    bool hasData = false;
    void* d = nullptr;           // one allocation, levels back to back
    size_t capacity = 0, used = 0;
    int levels = 0, storage = 0;
    size_t bytes[3] = {0, 0, 0};
    size_t wmBytes[3][4] = {};
    LevelDims dims[3];

    void release() {
        if (d) cudaFree(d);
        d = nullptr;
        capacity = used = 0;
        hasData = false;
    }
};

extern "C" fcfd_vram_snapshot* fcfd_vram_snapshot_create(void) { return new fcfd_vram_snapshot(); }

extern "C" void fcfd_vram_snapshot_destroy(fcfd_vram_snapshot* v) {
    if (!v) return;
    v->release();
    delete v;
}

extern "C" int fcfd_vram_snapshot_capture(fcfd_vram_snapshot* v, fcfd_solver* s, const fcfd_snapshot_key* key,
                                          char* err, size_t errlen) {
    if (!v || !s) return -1;
    SolverFieldView fv;
    if (solver_field_view(s, &fv) != 0) {
        say(err, errlen, "solver holds no field to capture");
        return -1;
    }
    size_t need = 0;
    for (int l = 0; l < fv.levels; ++l) {
        need += fv.bytes[l];
        for (int k = 0; k < 4; ++k) need += fv.wmBytes[l][k];
    }
    if (!v->d || v->capacity < need) {
        v->release();
        if (auto e = cudaMalloc(&v->d, need); e != cudaSuccess) {
            v->d = nullptr;
            say(err, errlen, std::string("VRAM snapshot allocation failed: ") + cudaGetErrorString(e));
            return static_cast<int>(e);
        }
        v->capacity = need;
    }
    size_t off = 0;
    auto copy = [&](const void* src, size_t b) {
        const cudaError_t e =
            b ? cudaMemcpyAsync(static_cast<char*>(v->d) + off, src, b, cudaMemcpyDeviceToDevice, fv.stream)
              : cudaSuccess;
        off += b;
        return e;
    };
    for (int l = 0; l < fv.levels; ++l) {
        cudaError_t e = copy(fv.f[l], fv.bytes[l]);
        for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = copy(fv.wm[l][k], fv.wmBytes[l][k]);
        if (e != cudaSuccess) {
            v->hasData = false;
            say(err, errlen, std::string("VRAM snapshot copy failed: ") + cudaGetErrorString(e));
            return static_cast<int>(e);
        }
        v->bytes[l] = fv.bytes[l];
        for (int k = 0; k < 4; ++k) v->wmBytes[l][k] = fv.wmBytes[l][k];
        v->dims[l] = fv.dims[l];
    }
    v->used = need;
    v->levels = fv.levels;
    v->storage = fv.storage;
    v->key = Key::of(key);
    v->flagsHash = fv.flagsHash;
    v->hasData = true;
    say(err, errlen, "");
    return 0;
}

extern "C" int fcfd_vram_snapshot_restore(const fcfd_vram_snapshot* v, fcfd_solver* s) {
    if (!v || !s || !v->hasData) return -1;
    SolverFieldView fv;
    if (solver_field_view(s, &fv) != 0) return -1;
    if (fv.levels != v->levels || fv.storage != v->storage) return -1;
    for (int l = 0; l < fv.levels; ++l) {
        if (fv.bytes[l] != v->bytes[l] || fv.dims[l].nx != v->dims[l].nx || fv.dims[l].ny != v->dims[l].ny
            || fv.dims[l].nz != v->dims[l].nz)
            return -1;
        for (int k = 0; k < 4; ++k)
            if (fv.wmBytes[l][k] != v->wmBytes[l][k]) return -1;
    }
    size_t off = 0;
    auto copy = [&](void* dst, size_t b) {
        const cudaError_t e =
            b ? cudaMemcpyAsync(dst, static_cast<const char*>(v->d) + off, b, cudaMemcpyDeviceToDevice, fv.stream)
              : cudaSuccess;
        off += b;
        return e;
    };
    for (int l = 0; l < fv.levels; ++l) {
        cudaError_t e = copy(fv.f[l], fv.bytes[l]);
        for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = copy(fv.wm[l][k], fv.wmBytes[l][k]);
        if (e != cudaSuccess) return static_cast<int>(e);
    }
    fcfd_notify_restored(s, 1);
    return 0;
}

extern "C" int fcfd_vram_snapshot_has_data(const fcfd_vram_snapshot* v) { return v && v->hasData ? 1 : 0; }
extern "C" uint64_t fcfd_vram_snapshot_flags_hash(const fcfd_vram_snapshot* v) { return v ? v->flagsHash : 0; }
extern "C" size_t fcfd_vram_snapshot_bytes(const fcfd_vram_snapshot* v) { return v && v->hasData ? v->used : 0; }
extern "C" int fcfd_vram_snapshot_key(const fcfd_vram_snapshot* v, fcfd_snapshot_key* key) {
    if (!v || !key || !v->hasData) return -1;
    v->key.out(key);
    return 0;
}
extern "C" void fcfd_vram_snapshot_release(fcfd_vram_snapshot* v) {
    if (v) v->release();
}

// ---- compact snapshot ------------------------------------------------------------

struct fcfd_compact_snapshot {
    Key key;
    std::uint64_t flagsHash = 0;
    fcfd_scaling scaling{};
    bool hasData = false;
    std::vector<float> rho, u, v, w;
};

namespace {

template <class T>
void put(std::ofstream& os, const T& x) {
    os.write(reinterpret_cast<const char*>(&x), sizeof(T));
}
template <class T>
bool get(std::ifstream& is, T& x) {
    is.read(reinterpret_cast<char*>(&x), sizeof(T));
    return static_cast<bool>(is);
}

bool save_fcs(const fcfd_compact_snapshot& c, const fs::path& path, std::string& why) {
    std::ofstream os(path, std::ios::binary | std::ios::trunc);
    if (!os) {
        why = "cannot open " + path.string() + " for writing";
        return false;
    }
    put(os, kFcsMagic);
    put(os, kFcsFormat);
    const auto idLen = static_cast<std::uint32_t>(c.key.id.size());
    put(os, idLen);
    os.write(c.key.id.data(), idLen);
    put(os, c.key.bucket);
    put(os, c.key.uLat);
    put(os, c.key.dims.nx);
    put(os, c.key.dims.ny);
    put(os, c.key.dims.nz);
    put(os, c.key.version);
    put(os, c.flagsHash);
    const fcfd_scaling& s = c.scaling;
    put(os, s.chord_m);
    put(os, s.airspeed_ms);
    put(os, s.nu_m2s);
    put(os, s.chord_cells);
    put(os, s.u_lat);
    put(os, s.dx);
    put(os, s.dt);
    put(os, s.nu_lat_target);
    put(os, s.nu_lat);
    put(os, s.tau);
    put(os, static_cast<std::uint8_t>(s.tau_clamped ? 1 : 0));
    put(os, s.re_target);
    put(os, s.re_effective);
    put(os, kPayloadRawF32);
    const auto n = static_cast<std::uint64_t>(c.rho.size());
    put(os, n);
    for (const std::vector<float>* a : {&c.rho, &c.u, &c.v, &c.w})
        os.write(reinterpret_cast<const char*>(a->data()), static_cast<std::streamsize>(a->size() * sizeof(float)));
    os.flush();
    if (!os) {
        why = "write failed (disk full?) at " + path.string();
        return false;
    }
    return true;
}

bool load_fcs(fcfd_compact_snapshot& c, const fs::path& path, std::string& why) {
    c.hasData = false;
    std::ifstream is(path, std::ios::binary);
    if (!is) {
        why = "cannot open " + path.string();
        return false;
    }
    auto bad = [&](const char* w) {
        why = std::string(w) + ": " + path.string();
        return false;
    };
    std::uint32_t magic = 0, format = 0, idLen = 0;
    if (!get(is, magic) || magic != kFcsMagic) return bad("bad magic");
    if (!get(is, format) || format != kFcsFormat) return bad("unsupported format version");
    if (!get(is, idLen) || idLen > kMaxIdBytes) return bad("corrupt geometry id");
    Key k;
    k.id.resize(idLen);
    if (idLen && !is.read(k.id.data(), idLen)) return bad("truncated header");
    if (!get(is, k.bucket) || !get(is, k.uLat) || !get(is, k.dims.nx) || !get(is, k.dims.ny) || !get(is, k.dims.nz)
        || !get(is, k.version))
        return bad("truncated header");
    if (k.version != FCFD_SOLVER_VERSION) return bad("solver version mismatch");
    std::uint64_t fh = 0;
    if (!get(is, fh)) return bad("truncated header");
    fcfd_scaling s{};
    std::uint8_t clamped = 0;
    const bool ok = get(is, s.chord_m) && get(is, s.airspeed_ms) && get(is, s.nu_m2s) && get(is, s.chord_cells)
                    && get(is, s.u_lat) && get(is, s.dx) && get(is, s.dt) && get(is, s.nu_lat_target)
                    && get(is, s.nu_lat) && get(is, s.tau) && get(is, clamped) && get(is, s.re_target)
                    && get(is, s.re_effective);
    if (!ok) return bad("truncated scaling block");
    s.tau_clamped = clamped ? 1 : 0;
    std::uint32_t payload = 0;
    std::uint64_t n = 0;
    if (!get(is, payload) || payload != kPayloadRawF32) return bad("unsupported payload compression");
    if (!get(is, n)) return bad("truncated payload header");
    // The count must be the key's own grid (a corrupt count would otherwise
    // size a huge allocation).
    const auto expect = static_cast<std::uint64_t>(k.dims.nx) * static_cast<std::uint64_t>(k.dims.ny)
                      * static_cast<std::uint64_t>(k.dims.nz);
    if (k.dims.nx <= 0 || k.dims.ny <= 0 || k.dims.nz <= 0 || n == 0 || n != expect)
        return bad("payload size mismatch");
    for (std::vector<float>* a : {&c.rho, &c.u, &c.v, &c.w}) {
        a->resize(static_cast<size_t>(n));
        if (!is.read(reinterpret_cast<char*>(a->data()), static_cast<std::streamsize>(n * sizeof(float))))
            return bad("truncated field payload");
    }
    c.key = k;
    c.flagsHash = fh;
    c.scaling = s;
    c.hasData = true;
    return true;
}

} // namespace

extern "C" fcfd_compact_snapshot* fcfd_compact_snapshot_create(void) { return new fcfd_compact_snapshot(); }
extern "C" void fcfd_compact_snapshot_destroy(fcfd_compact_snapshot* c) { delete c; }

extern "C" int fcfd_compact_snapshot_capture(fcfd_compact_snapshot* c, fcfd_solver* s, const fcfd_snapshot_key* key,
                                             char* err, size_t errlen) {
    if (!c || !s) return -1;
    SolverFieldView fv;
    if (solver_field_view(s, &fv) != 0) {
        say(err, errlen, "solver holds no field to capture");
        return -1;
    }
    const size_t n = static_cast<size_t>(fv.dims[0].cells());
    c->rho.resize(n); c->u.resize(n); c->v.resize(n); c->w.resize(n);
    if (auto e = fcfd_download_macro(s, c->rho.data(), c->u.data(), c->v.data(), c->w.data()); e != 0) {
        c->hasData = false;
        say(err, errlen, std::string("macroscopic download failed: ") + cudaGetErrorString(static_cast<cudaError_t>(e)));
        return e;
    }
    c->key = Key::of(key);
    c->scaling = fv.scaling;
    c->flagsHash = fv.flagsHash;
    c->hasData = true;
    say(err, errlen, "");
    return 0;
}

extern "C" int fcfd_compact_snapshot_restore(const fcfd_compact_snapshot* c, fcfd_solver* s) {
    if (!c || !s || !c->hasData) return -1;
    SolverFieldView fv;
    if (solver_field_view(s, &fv) != 0) return -1;
    if (fv.dims[0].nx != c->key.dims.nx || fv.dims[0].ny != c->key.dims.ny || fv.dims[0].nz != c->key.dims.nz
        || static_cast<size_t>(fv.dims[0].cells()) != c->rho.size())
        return -1;
    return fcfd_restore_from_macro(s, c->rho.data(), c->u.data(), c->v.data(), c->w.data());
}

extern "C" int fcfd_compact_snapshot_save(const fcfd_compact_snapshot* c, const char* path, char* err,
                                          size_t errlen) {
    if (!c || !path) return -1;
    if (!c->hasData) {
        say(err, errlen, "no snapshot data to save");
        return -1;
    }
    std::string why;
    if (!save_fcs(*c, path, why)) {
        say(err, errlen, why);
        return -1;
    }
    say(err, errlen, "");
    return 0;
}

extern "C" int fcfd_compact_snapshot_load(fcfd_compact_snapshot* c, const char* path, char* err, size_t errlen) {
    if (!c || !path) return -1;
    std::string why;
    if (!load_fcs(*c, path, why)) {
        say(err, errlen, why);
        return -1;
    }
    say(err, errlen, "");
    return 0;
}

extern "C" int fcfd_compact_snapshot_has_data(const fcfd_compact_snapshot* c) { return c && c->hasData ? 1 : 0; }
extern "C" uint64_t fcfd_compact_snapshot_flags_hash(const fcfd_compact_snapshot* c) { return c ? c->flagsHash : 0; }
extern "C" int fcfd_compact_snapshot_key(const fcfd_compact_snapshot* c, fcfd_snapshot_key* key) {
    if (!c || !key || !c->hasData) return -1;
    c->key.out(key);
    return 0;
}
extern "C" int fcfd_compact_snapshot_scaling(const fcfd_compact_snapshot* c, fcfd_scaling* scaling) {
    if (!c || !scaling || !c->hasData) return -1;
    *scaling = c->scaling;
    return 0;
}
extern "C" int fcfd_compact_snapshot_fields(const fcfd_compact_snapshot* c, const float** rho, const float** u,
                                            const float** v, const float** w, size_t* ncells) {
    if (!c || !c->hasData) return -1;
    if (rho) *rho = c->rho.data();
    if (u) *u = c->u.data();
    if (v) *v = c->v.data();
    if (w) *w = c->w.data();
    if (ncells) *ncells = c->rho.size();
    return 0;
}

// ---- disk cache ------------------------------------------------------------------

struct fcfd_disk_cache {
    fs::path dir;
    std::uint64_t budget = 0, used = 0;
    std::mutex m;                              // directory state
    std::mutex qm;                             // writer queue
    std::condition_variable qcv, idle;
    std::deque<fcfd_compact_snapshot*> queue;
    int inFlight = 0;
    bool stop = false;
    std::thread writer;

    static bool is_entry(const fs::directory_entry& e) {
        std::error_code ec;
        return e.is_regular_file(ec) && e.path().extension() == ".fcs";
    }
    void scan() {
        used = 0;
        std::error_code ec;
        for (const auto& e : fs::directory_iterator(dir, ec))
            if (is_entry(e)) used += static_cast<std::uint64_t>(e.file_size(ec));
    }
    /// Oldest-first eviction down to the budget; `keep` is never removed.
    void evict(const fs::path& keep) {
        while (used > budget) {
            std::error_code ec;
            fs::path victim;
            fs::file_time_type oldest = fs::file_time_type::max();
            std::uint64_t size = 0;
            for (const auto& e : fs::directory_iterator(dir, ec)) {
                if (!is_entry(e) || e.path() == keep) continue;
                const auto t = e.last_write_time(ec);
                if (t < oldest) {
                    oldest = t;
                    victim = e.path();
                    size = static_cast<std::uint64_t>(e.file_size(ec));
                }
            }
            if (victim.empty() || !fs::remove(victim, ec)) break;
            used = used > size ? used - size : 0;
        }
    }
    bool store(const fcfd_compact_snapshot& snap, std::string& why) {
        if (!snap.hasData) {
            why = "snapshot holds no data";
            return false;
        }
        std::lock_guard<std::mutex> lk(m);
        const std::string name = snap.key.fileName();
        const fs::path final = dir / name, tmp = dir / (name + ".tmp");
        std::error_code ec;
        if (!save_fcs(snap, tmp, why)) {
            fs::remove(tmp, ec);
            return false;
        }
        std::uint64_t replaced = 0;
        if (fs::exists(final, ec)) replaced = static_cast<std::uint64_t>(fs::file_size(final, ec));
        fs::rename(tmp, final, ec);
        if (ec) {
            why = "rename to " + final.string() + " failed: " + ec.message();
            fs::remove(tmp, ec);
            return false;
        }
        used = used - std::min(used, replaced) + static_cast<std::uint64_t>(fs::file_size(final, ec));
        evict(final);
        return true;
    }
    void writerLoop() {
        for (;;) {
            fcfd_compact_snapshot* snap = nullptr;
            {
                std::unique_lock<std::mutex> lk(qm);
                qcv.wait(lk, [this] { return stop || !queue.empty(); });
                if (queue.empty()) return;
                snap = queue.front();
                queue.pop_front();
                ++inFlight;
            }
            std::string why;
            if (!store(*snap, why)) std::fprintf(stderr, "[snapshot cache] background store failed: %s\n", why.c_str());
            delete snap;
            {
                std::lock_guard<std::mutex> lk(qm);
                --inFlight;
            }
            idle.notify_all();
        }
    }
};

extern "C" fcfd_disk_cache* fcfd_disk_cache_open(const char* directory, uint64_t budget_bytes) {
    if (!directory) return nullptr;
    auto* c = new fcfd_disk_cache();
    c->dir = directory;
    c->budget = budget_bytes;
    std::error_code ec;
    fs::create_directories(c->dir, ec);
    if (!fs::is_directory(c->dir, ec)) {
        delete c;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(c->m);
    c->scan();
    return c;
}

extern "C" void fcfd_disk_cache_close(fcfd_disk_cache* c) {
    if (!c) return;
    {
        std::lock_guard<std::mutex> lk(c->qm);
        c->stop = true;
    }
    c->qcv.notify_all();
    if (c->writer.joinable()) c->writer.join();
    for (auto* s : c->queue) delete s;
    delete c;
}

extern "C" int fcfd_disk_cache_find(fcfd_disk_cache* c, const fcfd_snapshot_key* key, char* path, size_t len) {
    if (!c || !key) return 0;
    std::lock_guard<std::mutex> lk(c->m);
    const fs::path p = c->dir / Key::of(key).fileName();
    std::error_code ec;
    if (!fs::exists(p, ec)) return 0;
    fs::last_write_time(p, fs::file_time_type::clock::now(), ec);   // a hit is recent use
    if (path && len) std::snprintf(path, len, "%s", p.string().c_str());
    return 1;
}

extern "C" int fcfd_disk_cache_store(fcfd_disk_cache* c, const fcfd_compact_snapshot* snap, char* err,
                                     size_t errlen) {
    if (!c || !snap) return -1;
    std::string why;
    if (!c->store(*snap, why)) {
        say(err, errlen, why);
        return -1;
    }
    say(err, errlen, "");
    return 0;
}

extern "C" int fcfd_disk_cache_store_async(fcfd_disk_cache* c, fcfd_compact_snapshot* snap) {
    if (!c || !snap) return -1;
    {
        std::lock_guard<std::mutex> lk(c->qm);
        if (!c->writer.joinable()) c->writer = std::thread([c] { c->writerLoop(); });
        c->queue.push_back(snap);
    }
    c->qcv.notify_one();
    return 0;
}

extern "C" void fcfd_disk_cache_wait(fcfd_disk_cache* c) {
    if (!c) return;
    std::unique_lock<std::mutex> lk(c->qm);
    c->idle.wait(lk, [c] { return c->queue.empty() && c->inFlight == 0; });
}

extern "C" void fcfd_disk_cache_set_budget(fcfd_disk_cache* c, uint64_t budget_bytes) {
    if (!c) return;
    std::lock_guard<std::mutex> lk(c->m);
    c->budget = budget_bytes;
    c->evict(fs::path());
}

extern "C" uint64_t fcfd_disk_cache_used_bytes(fcfd_disk_cache* c) {
    if (!c) return 0;
    std::lock_guard<std::mutex> lk(c->m);
    return c->used;
}
