// kv_standin.cpp -- a key/value store with the entry points the scene-file
// code loads from unqlite (unqlite_open / config / close / kv_store /
// kv_append / kv_fetch / kv_delete / commit / rollback), for tests on
// machines where the reference's unqlite source is absent.  Test
// infrastructure only: records live in a std::map, commit writes them to the
// file in this store's own format (not unqlite's): repeated
// [u32 key bytes][key][u64 value bytes][value].
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

namespace {

constexpr int OK = 0, NOTFOUND = -6, IOERR = -2;

struct Store {
    std::string path;
    std::map<std::string, std::string> kv;
};

bool load(Store* s) {
    s->kv.clear();
    FILE* f = std::fopen(s->path.c_str(), "rb");
    if (!f) return false;
    for (;;) {
        uint32_t kl;
        uint64_t vl;
        if (std::fread(&kl, sizeof kl, 1, f) != 1) break;
        std::string k(kl, '\0'), v;
        if (kl && std::fread(&k[0], 1, kl, f) != kl) break;
        if (std::fread(&vl, sizeof vl, 1, f) != 1) break;
        v.resize(vl);
        if (vl && std::fread(&v[0], 1, vl, f) != vl) break;
        s->kv[k] = v;
    }
    std::fclose(f);
    return true;
}

int save(Store* s) {
    FILE* f = std::fopen(s->path.c_str(), "wb");
    if (!f) return IOERR;
    for (auto& e : s->kv) {
        const uint32_t kl = (uint32_t)e.first.size();
        const uint64_t vl = e.second.size();
        std::fwrite(&kl, sizeof kl, 1, f);
        std::fwrite(e.first.data(), 1, kl, f);
        std::fwrite(&vl, sizeof vl, 1, f);
        std::fwrite(e.second.data(), 1, vl, f);
    }
    return std::fclose(f) == 0 ? OK : IOERR;
}

std::string key(const void* k, int n) { return std::string(static_cast<const char*>(k), (size_t)(n < 0 ? std::strlen(static_cast<const char*>(k)) : n)); }

}  // namespace

extern "C" {

int unqlite_open(void** db, const char* path, unsigned) {
    auto* s = new Store();
    s->path = path ? path : "";
    load(s);   // a missing file opens empty
    *db = s;
    return OK;
}

int unqlite_config(void*, int, ...) { return OK; }

int unqlite_close(void* db) {
    auto* s = static_cast<Store*>(db);
    const int rc = save(s);   // unqlite commits on close
    delete s;
    return rc;
}

int unqlite_kv_store(void* db, const void* k, int kn, const void* v, long long vn) {
    static_cast<Store*>(db)->kv[key(k, kn)] = std::string(static_cast<const char*>(v), (size_t)vn);
    return OK;
}

int unqlite_kv_append(void* db, const void* k, int kn, const void* v, long long vn) {
    static_cast<Store*>(db)->kv[key(k, kn)].append(static_cast<const char*>(v), (size_t)vn);
    return OK;
}

int unqlite_kv_fetch(void* db, const void* k, int kn, void* buf, long long* n) {
    auto& kv = static_cast<Store*>(db)->kv;
    auto it = kv.find(key(k, kn));
    if (it == kv.end()) return NOTFOUND;
    if (!buf) {
        *n = (long long)it->second.size();
        return OK;
    }
    const size_t m = std::min((size_t)*n, it->second.size());
    std::memcpy(buf, it->second.data(), m);
    *n = (long long)m;
    return OK;
}

int unqlite_kv_delete(void* db, const void* k, int kn) {
    return static_cast<Store*>(db)->kv.erase(key(k, kn)) ? OK : NOTFOUND;
}

int unqlite_commit(void* db) { return save(static_cast<Store*>(db)); }

int unqlite_rollback(void* db) {
    load(static_cast<Store*>(db));
    return OK;
}

}  // extern "C"
