// pstdfile.cpp -- openPSTD scene files (.pstd): the scene configuration and
// the results of a run in a key/value store, as shared/PSTDFile.cpp of the
// reference keeps them.
//
// File layout (shared/PSTDFile.cpp:50-60, 163-340, 404-453):
//   key = int32 prefix followed by int32 indices, stored as raw bytes
//   {10000}          int32 file version, 4
//   {1}              scene configuration (Boost text archive of PSTDConfiguration)
//   {100}            configuration the results were computed for (same encoding)
//   {102, d}         int32 number of frames saved for domain d
//   {103, d, f}      frame f of domain d: Nx*Ny float32, row-major (x fastest)
//   {104, r}         float32 samples of receiver r, appended as they arrive
// The store is unqlite (a single-file key/value engine the reference vendors
// and builds as a shared library); this module loads it at run time
// (dlopen of the library named by the caller or PSTD_UNQLITE_LIB, else
// "libunqlite.so") and never links it.
//
// The configuration encoding restates Boost.Serialization's text archive for
// the member order of PSTDConfiguration::serialize (kernel/KernelInterface.h:
// 80-97, 170-175, 196-205, 233-240) and the QVector2D / QVector3D free
// functions (shared/PSTDFile.h:63-111):
//   "22 serialization::archive <library version>", then, space separated,
//   for the first object of every class type its tracking level and version
//   ("0 0"), then its members in serialize order; float members with 9
//   significant digits; bool as 0 / 1; std::vector as its element count, the
//   element class version (library versions > 3) and the elements.
#include <dlfcn.h>

#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pstd_gb300.h"

namespace pstd {
namespace {

constexpr int kFileVersion = 4;
constexpr uint32_t kPrefixScene = 1, kPrefixResultsScene = 100, kPrefixFrameCount = 102, kPrefixFrameData = 103,
                   kPrefixReceiverData = 104, kPrefixVersion = 10000;
// Boost library version written into new archives (Boost 1.58 writes 12;
// every later reader accepts it)
constexpr int kArchiveLibraryVersion = 12;

struct FileError : std::runtime_error {
    int code;
    FileError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

thread_local std::string g_file_error;

// ---------------------------------------------------------------- archive
enum ClassId { C_CONF, C_SETTINGS, C_VEC3, C_VEC2, C_DOMAIN, C_EDGE, C_COUNT };

struct Writer {
    std::string out;
    bool seen[C_COUNT] = {};
    void tok(const std::string& s) {
        if (!out.empty()) out += ' ';
        out += s;
    }
    void i(long long v) { tok(std::to_string(v)); }
    void f(float v) {
        char b[48];
        std::snprintf(b, sizeof b, "%.9g", (double)v);
        tok(b);
    }
    void cls(ClassId c) {   // tracking level and class version, first object of a class only
        if (seen[c]) return;
        seen[c] = true;
        i(0);
        i(0);
    }
    void collection(long long n) {
        i(n);
        i(0);   // element class version
    }
};

std::string encode(const pstd_config& c) {
    Writer w;
    w.i(22);
    w.tok("serialization::archive");
    w.i(kArchiveLibraryVersion);
    w.cls(C_CONF);
    w.cls(C_SETTINGS);
    const pstd_settings& s = c.settings;
    for (float v : {s.calctime, s.c1, s.ampMax, s.freqMax, s.rho, s.patcherror, s.tfactRK, s.gridSpacing, s.band_width,
                    s.wave_length})
        w.f(v);
    const int nrk = s.n_rk_coefficients < 0 ? 0 : (s.n_rk_coefficients > 6 ? 6 : s.n_rk_coefficients);
    w.collection(nrk);
    for (int k = 0; k < nrk; k++) w.f(s.rk_coefficients[k]);
    w.i(s.spectral_interpolation ? 1 : 0);
    w.i(s.PMLCells);
    w.i(s.SaveNth);
    for (int which = 0; which < 2; which++) {
        const int n = which ? c.n_receivers : c.n_speakers;
        const float* p = which ? c.receivers : c.speakers;
        w.collection(n);
        for (int k = 0; k < n; k++) {
            w.cls(C_VEC3);
            for (int e = 0; e < 3; e++) w.f(p[3 * k + e]);
        }
    }
    w.collection(c.n_domains);
    for (int k = 0; k < c.n_domains; k++) {
        const pstd_domain_conf& d = c.domains[k];
        w.cls(C_DOMAIN);
        w.cls(C_VEC2);
        w.f(d.top_left[0]);
        w.f(d.top_left[1]);
        w.f(d.size[0]);
        w.f(d.size[1]);
        for (const pstd_domain_edge* e : {&d.T, &d.L, &d.B, &d.R}) {
            w.cls(C_EDGE);
            w.f(e->absorption);
            w.i(e->lr ? 1 : 0);
        }
    }
    w.out += '\n';
    return w.out;
}

// A decoded configuration and the arrays its pstd_config points into.
struct Decoded {
    pstd_config c{};
    std::vector<pstd_domain_conf> domains;
    std::vector<float> speakers, receivers;
    void bind() {
        c.n_domains = (int32_t)domains.size();
        c.domains = domains.data();
        c.n_speakers = (int32_t)(speakers.size() / 3);
        c.speakers = speakers.data();
        c.n_receivers = (int32_t)(receivers.size() / 3);
        c.receivers = receivers.data();
    }
};

struct Reader {
    const char* p;
    const char* end;
    int libver = 0;
    bool seen[C_COUNT] = {};
    std::string next() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t' || *p == 0)) p++;
        const char* s = p;
        while (p < end && !(*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t' || *p == 0)) p++;
        if (s == p) throw FileError(PSTD_ERR_INVALID, "scene archive ends early");
        return std::string(s, p);
    }
    long long i() {
        const std::string t = next();
        char* e = nullptr;
        errno = 0;
        const long long v = std::strtoll(t.c_str(), &e, 10);
        if (errno || !e || *e) throw FileError(PSTD_ERR_INVALID, "scene archive: '" + t + "' is not an integer");
        return v;
    }
    float f() {
        const std::string t = next();
        char* e = nullptr;
        const float v = std::strtof(t.c_str(), &e);
        if (!e || *e) throw FileError(PSTD_ERR_INVALID, "scene archive: '" + t + "' is not a number");
        return v;
    }
    void cls(ClassId c) {
        if (seen[c]) return;
        seen[c] = true;
        const long long tracking = i();
        i();   // class version (all versions of these classes share one layout)
        if (tracking != 0)
            throw FileError(PSTD_ERR_UNSUPPORTED, "scene archive: tracked objects are not supported");
    }
    long long collection(long long cap) {
        const long long n = i();
        if (libver > 3) i();   // element class version
        if (n < 0 || n > cap) throw FileError(PSTD_ERR_INVALID, "scene archive: collection size out of range");
        return n;
    }
};

void decode(const char* text, size_t n, Decoded& out) {
    Reader r{text, text + n};
    if (r.i() != 22 || r.next() != "serialization::archive")
        throw FileError(PSTD_ERR_INVALID, "not a Boost text archive (no 'serialization::archive' header)");
    r.libver = (int)r.i();
    r.cls(C_CONF);
    r.cls(C_SETTINGS);
    pstd_settings& s = out.c.settings;
    std::memset(&s, 0, sizeof s);
    float* fs[] = {&s.calctime, &s.c1, &s.ampMax, &s.freqMax, &s.rho, &s.patcherror, &s.tfactRK, &s.gridSpacing,
                   &s.band_width, &s.wave_length};
    for (float* v : fs) *v = r.f();
    const long long nrk = r.collection(1 << 20);
    if (nrk > 6) throw FileError(PSTD_ERR_UNSUPPORTED, "scene archive: more than 6 Runge-Kutta coefficients");
    s.n_rk_coefficients = (int32_t)nrk;
    for (long long k = 0; k < nrk; k++) s.rk_coefficients[k] = r.f();
    s.spectral_interpolation = (int32_t)r.i();
    s.PMLCells = (int32_t)r.i();
    s.SaveNth = (int32_t)r.i();
    for (int which = 0; which < 2; which++) {
        std::vector<float>& v = which ? out.receivers : out.speakers;
        const long long m = r.collection(1 << 24);
        v.resize((size_t)m * 3);
        for (long long k = 0; k < m; k++) {
            r.cls(C_VEC3);
            for (int e = 0; e < 3; e++) v[(size_t)k * 3 + e] = r.f();
        }
    }
    const long long nd = r.collection(1 << 24);
    out.domains.resize((size_t)nd);
    for (long long k = 0; k < nd; k++) {
        pstd_domain_conf& d = out.domains[(size_t)k];
        r.cls(C_DOMAIN);
        r.cls(C_VEC2);
        d.top_left[0] = r.f();
        d.top_left[1] = r.f();
        d.size[0] = r.f();
        d.size[1] = r.f();
        for (pstd_domain_edge* e : {&d.T, &d.L, &d.B, &d.R}) {
            r.cls(C_EDGE);
            e->absorption = r.f();
            e->lr = (int32_t)r.i();
        }
    }
    out.bind();
}

// PSTDConfiguration::CreateDefaultConf (kernel/KernelInterface.cpp:196-249)
// and CreateEmptyConf (:251-268); members the reference leaves unset are 0
void default_config(Decoded& d) {
    pstd_settings& s = d.c.settings;
    std::memset(&s, 0, sizeof s);
    s.calctime = 1.0f;
    s.c1 = 340.0f;
    s.ampMax = 20000.0f;
    s.rho = 1.2f;
    s.patcherror = 70.0f;
    s.tfactRK = 0.5f;
    s.gridSpacing = 0.2f;
    s.PMLCells = 50;
    s.SaveNth = 1;
    const float q = 340.0f / 0.2f;
    s.band_width = (float)(3 * 1e-6 * q * q);
    const float rk[6] = {1.179799016570605e-1f, 1.846469664911166e-1f, 2.466236043095944e-1f,
                         3.318395427360000e-1f, 5e-1f, 1.0f};
    for (int k = 0; k < 6; k++) s.rk_coefficients[k] = rk[k];
    s.n_rk_coefficients = 6;
    s.spectral_interpolation = 1;
    d.speakers = {4, 5, 0};
    d.receivers = {6, 5, 0};
    pstd_domain_conf a{}, b{};
    a.top_left[0] = 0; a.top_left[1] = 0; a.size[0] = 10; a.size[1] = 15;
    a.T.absorption = 1; a.B.absorption = 0; a.L.absorption = 0.3f; a.R.absorption = 1;
    b.top_left[0] = 10; b.top_left[1] = 4; b.size[0] = 20; b.size[1] = 15;
    b.T.absorption = 1; b.B.absorption = 0; b.L.absorption = 1; b.R.absorption = 1;
    d.domains = {a, b};
    d.bind();
}

void empty_config(Decoded& d) {
    std::memset(&d.c.settings, 0, sizeof d.c.settings);
    d.domains.clear();
    d.speakers.clear();
    d.receivers.clear();
    d.bind();
}

// ---------------------------------------------------------------- store
constexpr int UQ_OK = 0, UQ_NOTFOUND = -6;
constexpr unsigned UQ_OPEN_CREATE = 0x4;
constexpr int UQ_CONFIG_DISABLE_AUTO_COMMIT = 5;

struct Unqlite {
    void* lib = nullptr;
    int (*open)(void**, const char*, unsigned) = nullptr;
    int (*config)(void*, int, ...) = nullptr;
    int (*close)(void*) = nullptr;
    int (*store)(void*, const void*, int, const void*, long long) = nullptr;
    int (*append)(void*, const void*, int, const void*, long long) = nullptr;
    int (*fetch)(void*, const void*, int, void*, long long*) = nullptr;
    int (*remove)(void*, const void*, int) = nullptr;
    int (*commit)(void*) = nullptr;
    int (*rollback)(void*) = nullptr;

    void load(const char* path) {
        std::string name = path && *path ? path : "";
        if (name.empty()) {
            const char* e = std::getenv("PSTD_UNQLITE_LIB");
            name = e && *e ? e : "libunqlite.so";
        }
        lib = dlopen(name.c_str(), RTLD_NOW | RTLD_LOCAL);
        if (!lib)
            throw FileError(PSTD_ERR_UNSUPPORTED, "cannot load the unqlite library '" + name + "' (" + dlerror() +
                                                      "): build shared/unqlite (libunqlite.so) and pass its path or "
                                                      "set PSTD_UNQLITE_LIB");
        auto sym = [&](const char* s) {
            void* f = dlsym(lib, s);
            if (!f) throw FileError(PSTD_ERR_UNSUPPORTED, std::string("unqlite library lacks ") + s);
            return f;
        };
        open = reinterpret_cast<decltype(open)>(sym("unqlite_open"));
        config = reinterpret_cast<decltype(config)>(sym("unqlite_config"));
        close = reinterpret_cast<decltype(close)>(sym("unqlite_close"));
        store = reinterpret_cast<decltype(store)>(sym("unqlite_kv_store"));
        append = reinterpret_cast<decltype(append)>(sym("unqlite_kv_append"));
        fetch = reinterpret_cast<decltype(fetch)>(sym("unqlite_kv_fetch"));
        remove = reinterpret_cast<decltype(remove)>(sym("unqlite_kv_delete"));
        commit = reinterpret_cast<decltype(commit)>(sym("unqlite_commit"));
        rollback = reinterpret_cast<decltype(rollback)>(sym("unqlite_rollback"));
    }
    ~Unqlite() {
        if (lib) dlclose(lib);
    }
};

using Key = std::vector<uint32_t>;

std::string key_text(const Key& k) {   // {prefix,[i,j]} as PSTDFileKeyToString prints it
    std::string s = "{" + std::to_string(k[0]) + ",[";
    for (size_t i = 1; i < k.size(); i++) s += (i > 1 ? "," : "") + std::to_string(k[i]);
    return s + "]}";
}

}  // namespace

struct PstdFile {
    Unqlite uq;
    void* db = nullptr;
    Decoded scene, results;   // backing of the configurations handed out

    void check(int rc, const Key* k, const char* action) const {
        if (rc == UQ_OK) return;
        std::string m = std::string("unqlite error ") + std::to_string(rc) + " on '" + action + "'";
        if (k) m += " with key " + key_text(*k);
        throw FileError(rc == UQ_NOTFOUND ? PSTD_ERR_INVALID : PSTD_ERR_IO, m);
    }
    void put(const Key& k, const void* data, long long n) {
        check(uq.store(db, k.data(), (int)(k.size() * 4), data, n), &k, "store data");
    }
    void add(const Key& k, const void* data, long long n) {
        check(uq.append(db, k.data(), (int)(k.size() * 4), data, n), &k, "append data");
    }
    std::vector<char> get(const Key& k) {
        long long n = 0;
        check(uq.fetch(db, k.data(), (int)(k.size() * 4), nullptr, &n), &k, "fetch data");
        std::vector<char> buf((size_t)n);
        if (n) check(uq.fetch(db, k.data(), (int)(k.size() * 4), buf.data(), &n), &k, "fetch data");
        buf.resize((size_t)n);
        return buf;
    }
    bool has(const Key& k) {
        long long n = 0;
        return uq.fetch(db, k.data(), (int)(k.size() * 4), nullptr, &n) == UQ_OK;
    }
    void del(const Key& k) { check(uq.remove(db, k.data(), (int)(k.size() * 4)), &k, "delete data"); }
    int get_int(const Key& k) {
        auto b = get(k);
        if (b.size() != 4) throw FileError(PSTD_ERR_INVALID, "record " + key_text(k) + " is not one int32");
        int v;
        std::memcpy(&v, b.data(), 4);
        return v;
    }
    void put_int(const Key& k, int v) { put(k, &v, 4); }
    void put_conf(const Key& k, const pstd_config& c) {
        const std::string s = encode(c);
        put(k, s.data(), (long long)s.size());
    }
    void get_conf(const Key& k, Decoded& d) {
        auto b = get(k);
        decode(b.data(), b.size(), d);
    }

    // PSTDFile::InitializeResults (shared/PSTDFile.cpp:234-249)
    void initialize_results() {
        Decoded sc;
        get_conf({kPrefixScene}, sc);
        put_conf({kPrefixResultsScene}, sc.c);
        for (uint32_t d = 0; d < sc.domains.size(); d++) put_int({kPrefixFrameCount, d}, 0);
        for (uint32_t r = 0; r < sc.receivers.size() / 3; r++) put({kPrefixReceiverData, r}, nullptr, 0);
    }
    // PSTDFile::DeleteResults (shared/PSTDFile.cpp:251-266)
    void delete_results() {
        Decoded rs;
        get_conf({kPrefixResultsScene}, rs);
        for (uint32_t d = 0; d < rs.domains.size(); d++) {
            const Key fc{kPrefixFrameCount, d};
            if (!has(fc)) continue;
            const int frames = get_int(fc);
            for (uint32_t f = 0; f < (uint32_t)frames; f++) del({kPrefixFrameData, d, f});
            del(fc);
        }
        Decoded e;
        empty_config(e);
        put_conf({kPrefixResultsScene}, e.c);
    }
};

}  // namespace pstd

using pstd::FileError;
using pstd::PstdFile;

#define FILE_GUARD(...)                                          \
    try {                                                        \
        __VA_ARGS__                                              \
    } catch (FileError & e) {                                    \
        pstd::g_file_error = e.what();                           \
        return e.code;                                           \
    } catch (std::exception & e) {                               \
        pstd::g_file_error = e.what();                           \
        return PSTD_ERR_INVALID;                                 \
    }

extern "C" {

const char* pstd_file_last_error(void) { return pstd::g_file_error.c_str(); }

int pstd_archive_encode(const pstd_config* config, char* buf, int64_t cap, int64_t* len) {
    FILE_GUARD({
        if (!config || !len) throw FileError(PSTD_ERR_INVALID, "config or len is NULL");
        const std::string s = pstd::encode(*config);
        *len = (int64_t)s.size();
        if (buf && cap > 0) {
            const size_t n = std::min<size_t>((size_t)cap - 1, s.size());
            std::memcpy(buf, s.data(), n);
            buf[n] = 0;
        }
        return PSTD_OK;
    })
}

int pstd_file_open(const char* path, const char* unqlite_lib, int32_t create_new, pstd_file** out) {
    FILE_GUARD({
        if (!path || !out) throw FileError(PSTD_ERR_INVALID, "path or out is NULL");
        *out = nullptr;
        auto f = std::make_unique<PstdFile>();
        f->uq.load(unqlite_lib);
        f->check(f->uq.open(&f->db, path, pstd::UQ_OPEN_CREATE), nullptr, "open");
        f->check(f->uq.config(f->db, pstd::UQ_CONFIG_DISABLE_AUTO_COMMIT), nullptr, "configure");
        if (create_new) {
            // PSTDFile::New (shared/PSTDFile.cpp:183-205)
            f->put_int({pstd::kPrefixVersion}, pstd::kFileVersion);
            pstd::Decoded d, e;
            pstd::default_config(d);
            pstd::empty_config(e);
            f->put_conf({pstd::kPrefixScene}, d.c);
            f->put_conf({pstd::kPrefixResultsScene}, e.c);
            f->check(f->uq.commit(f->db), nullptr, "Commit");
        } else {
            // PSTDFile::Open (shared/PSTDFile.cpp:168-181)
            if (!f->has({pstd::kPrefixVersion}))
                throw FileError(PSTD_ERR_INVALID, std::string(path) + " is not a PSTD file (no version record)");
            const int v = f->get_int({pstd::kPrefixVersion});
            if (v != pstd::kFileVersion)
                throw FileError(PSTD_ERR_UNSUPPORTED, "Wrong version: " + std::to_string(v) +
                                                          "(expected: " + std::to_string(pstd::kFileVersion) + ")");
        }
        *out = reinterpret_cast<pstd_file*>(f.release());
        return PSTD_OK;
    })
}

void pstd_file_close(pstd_file* h) {
    auto* f = reinterpret_cast<PstdFile*>(h);
    if (!f) return;
    if (f->db) f->uq.close(f->db);   // unqlite_close commits pending changes
    delete f;
}

int pstd_file_get_scene(pstd_file* h, int32_t results, pstd_config* out) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || !out) throw FileError(PSTD_ERR_INVALID, "file or out is NULL");
        pstd::Decoded& d = results ? f->results : f->scene;
        d = pstd::Decoded();
        f->get_conf({results ? pstd::kPrefixResultsScene : pstd::kPrefixScene}, d);
        *out = d.c;
        return PSTD_OK;
    })
}

int pstd_file_set_scene(pstd_file* h, int32_t results, const pstd_config* config) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || !config) throw FileError(PSTD_ERR_INVALID, "file or config is NULL");
        f->put_conf({results ? pstd::kPrefixResultsScene : pstd::kPrefixScene}, *config);
        return PSTD_OK;
    })
}

int pstd_file_initialize_results(pstd_file* h) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f) throw FileError(PSTD_ERR_INVALID, "file is NULL");
        f->initialize_results();
        return PSTD_OK;
    })
}

int pstd_file_delete_results(pstd_file* h) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f) throw FileError(PSTD_ERR_INVALID, "file is NULL");
        f->delete_results();
        return PSTD_OK;
    })
}

int pstd_file_save_frame(pstd_file* h, int32_t domain, const float* data, int64_t n) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || (n && !data) || domain < 0 || n < 0) throw FileError(PSTD_ERR_INVALID, "bad frame arguments");
        // PSTDFile::SaveNextResultsFrame / IncrementFrameCount (shared/PSTDFile.cpp:227-232, 444-450)
        const pstd::Key fc{pstd::kPrefixFrameCount, (uint32_t)domain};
        const int frame = f->get_int(fc);
        f->put_int(fc, frame + 1);
        f->put({pstd::kPrefixFrameData, (uint32_t)domain, (uint32_t)frame}, data, n * (int64_t)sizeof(float));
        return PSTD_OK;
    })
}

int pstd_file_frame_count(pstd_file* h, int32_t domain, int32_t* count) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || !count || domain < 0) throw FileError(PSTD_ERR_INVALID, "bad arguments");
        *count = f->get_int({pstd::kPrefixFrameCount, (uint32_t)domain});
        return PSTD_OK;
    })
}

int pstd_file_get_frame(pstd_file* h, int32_t domain, int32_t frame, float* dst, int64_t cap, int64_t* n) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || !n || domain < 0 || frame < 0) throw FileError(PSTD_ERR_INVALID, "bad arguments");
        const auto b = f->get({pstd::kPrefixFrameData, (uint32_t)domain, (uint32_t)frame});
        *n = (int64_t)(b.size() / 4);
        if (dst) std::memcpy(dst, b.data(), (size_t)std::min<int64_t>(cap, *n) * 4);
        return PSTD_OK;
    })
}

int pstd_file_append_samples(pstd_file* h, int32_t receiver, const float* data, int64_t n) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || (n && !data) || receiver < 0 || n < 0) throw FileError(PSTD_ERR_INVALID, "bad sample arguments");
        // PSTDFile::SaveReceiverData (shared/PSTDFile.cpp:481-485)
        f->add({pstd::kPrefixReceiverData, (uint32_t)receiver}, data, n * (int64_t)sizeof(float));
        return PSTD_OK;
    })
}

int pstd_file_get_samples(pstd_file* h, int32_t receiver, float* dst, int64_t cap, int64_t* n) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f || !n || receiver < 0) throw FileError(PSTD_ERR_INVALID, "bad arguments");
        const auto b = f->get({pstd::kPrefixReceiverData, (uint32_t)receiver});
        *n = (int64_t)(b.size() / 4);
        if (dst) std::memcpy(dst, b.data(), (size_t)std::min<int64_t>(cap, *n) * 4);
        return PSTD_OK;
    })
}

int pstd_file_commit(pstd_file* h) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f) throw FileError(PSTD_ERR_INVALID, "file is NULL");
        f->check(f->uq.commit(f->db), nullptr, "Commit");
        return PSTD_OK;
    })
}

int pstd_file_rollback(pstd_file* h) {
    FILE_GUARD({
        auto* f = reinterpret_cast<PstdFile*>(h);
        if (!f) throw FileError(PSTD_ERR_INVALID, "file is NULL");
        f->check(f->uq.rollback(f->db), nullptr, "Rollback");
        return PSTD_OK;
    })
}

}  // extern "C"
