// server.cu -- the serving loop: continuous batching of scene solves on one
// GPU (include/pstd_gb300.h, pstd_server_*).
//
// Requests (a scene and a step count) are built on the host at submit time,
// queue, and are admitted -- in arrival order -- when their fields fit the
// device arenas (admission by HBM footprint).  All admitted scenes form one
// batch, run in one of two forms.
//
// Persistent form (every strip length of the batch is one the merged kernel
// handles, 128 .. 2048; stage_all.cu): every RK stage is ONE launch of the
// merged persistent kernel over the strip jobs of all active scenes, and the
// stage, PML and receiver launches read their counts from device memory.  The
// domain table and two job tables (transform length >= 1024, taken first,
// and the rest) are arenas: a scene's entries are written once when it is
// admitted and zeroed (skipped by the kernel) when it leaves; the PML list,
// receivers, slots and counts are rewritten in place on the server's stream.
// The three step graphs are therefore captured once and replay unchanged;
// only a table that outgrows its capacity (it doubles) or a change of form
// captures them again.  Each scene has a step limit on the device: a tick
// runs up to max_steps steps, and a scene that reaches its count stops there
// (its jobs, PML pass and receiver samples are skipped) until the tick ends.
//
// Per-length form (other lengths, PSTD_VARIANT, or PSTD_SERVE_PERSISTENT=0):
// the stage kernel once per strip-length bucket with tuned variants (the
// batched plan of pstd_create_batch), tables and graphs built afresh per
// membership, and a tick advances every scene by the same number of steps, no
// further than the scene closest to completion.
//
// After a tick, finished scenes hand their receiver series (and optionally the
// last frame) to the host and free their ranges, and waiting requests are
// admitted into the freed space.  Scenes that join later run in the same
// launches as the ones already running: their work overlaps on the device.
//
// Device memory is reserved once (the budget): three state-set arenas of equal
// layout (a scene has the same offset in all three), the fixed-buffer arena of
// rigid domains, the p0 arena and an auxiliary arena for receiver rings.  The
// results of a scene do not depend on the other scenes of the batch: every
// strip job reads and writes only its own scene's fields.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pstd_gb300.h"
#include "kernel_state.hpp"

namespace pstd {

// first-fit allocator of ranges: offsets and lengths in units (floats of an
// arena, entries of a table), lengths rounded up to multiples of `gran`
struct RangeAlloc {
    size_t cap = 0, used = 0, peak = 0, gran = 64;
    std::map<size_t, size_t> free_;   // offset -> length

    size_t round(size_t n) const { return (std::max<size_t>(n, 1) + gran - 1) / gran * gran; }
    void init(size_t c, size_t g = 64) {
        gran = g;
        cap = c / gran * gran;
        used = peak = 0;
        free_.clear();
        if (cap) free_[0] = cap;
    }
    bool alloc(size_t n, size_t* off) {
        n = round(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const size_t rest = it->second - n, o2 = it->first + n;
            free_.erase(it);
            if (rest) free_[o2] = rest;
            used += n;
            peak = std::max(peak, used);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t n) {
        n = round(n);
        used -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    // end of the highest range in use
    size_t top() const {
        if (free_.empty()) return cap;
        const auto last = std::prev(free_.end());
        return last->first + last->second == cap ? last->first : cap;
    }
    // capacity c > cap: the new units are free
    void grow(size_t c) {
        c = c / gran * gran;
        if (c <= cap) return;
        const size_t old = cap, extra = c - cap;
        cap = c;
        used += extra;
        release(old, extra);
    }
};

struct Request {
    int64_t id = 0;
    int n_steps = 0, flags = 0;
    int state = PSTD_REQ_QUEUED;
    int steps_done = 0;
    Scene scene;
    std::vector<DevDomain> local;                        // offsets relative to the scene's ranges
    size_t set_f = 0, fixed_f = 0, p0_f = 0, aux_f = 0;  // floats per arena
    size_t set_off = 0, fixed_off = 0, p0_off = 0, aux_off = 0;
    int slot = -1;
    int64_t cells = 0;                                   // non-rigid cells (work per step)
    int64_t frame_f = 0;                                 // non-PML cells (final frame)
    std::vector<float> receivers, frame;                 // results, step-major
    std::string error;
    // persistent form: the scene's strip lengths, its strip jobs by transform
    // length (key 0: copy jobs; domain indices local to the scene) for the
    // configuration set `jobs_set`, and its ranges in the domain table and
    // the job regions ((region, offset) per entry of `jobs`, same order)
    std::vector<int> lengths;
    int jobs_set = -1;
    std::map<int, std::vector<DevJob>> jobs;
    bool placed = false;
    size_t dom_off = 0;
    std::vector<std::pair<int, size_t>> job_ranges;
    int final_set = 0;                                   // state set holding the last step

    int64_t bytes() const { return (int64_t)(3 * set_f + fixed_f + p0_f + aux_f) * 4; }
};

// Field layout of one scene relative to its own ranges (the layout pstd_create
// uses, Kernel::layout_domain); attenuation profiles are shared across
// requests through one table.
static void layout_scene(Request& q, std::vector<float>& att, std::map<std::tuple<int, int, int, float, float, float>, int>& att_off) {
    const Scene& sc = q.scene;
    long long off = 0, foff = 0, poff = 0;
    q.local.assign(sc.doms.size(), DevDomain{});
    q.cells = 0;
    q.frame_f = 0;
    for (size_t k = 0; k < sc.doms.size(); k++) {
        const Domain& d = sc.doms[k];
        DevDomain& h = q.local[k];
        Kernel::layout_domain(d, sc, 0, off, foff, poff, h);
        if (d.pml) {
            // profiles depend on (PML cells, velocity, ascending, ampMax, dt, rho): shared across requests
            const float dt = sc.s.dt();
            auto put = [&](bool vel, bool asc, int& at) {
                auto key = std::make_tuple(sc.s.pml_cells, (int)vel, (int)asc, sc.s.ampMax, dt, sc.s.rho);
                auto it = att_off.find(key);
                if (it != att_off.end()) { at = it->second; return; }
                std::vector<double> prof;
                pml_profile(sc.s, vel, asc, prof);
                at = (int)att.size();
                for (double v : prof) att.push_back((float)v);
                att_off[key] = at;
            };
            if (d.att_x) { put(false, d.asc_x, h.att_xp); put(true, d.asc_x, h.att_xv); }
            if (d.att_y) { put(false, d.asc_y, h.att_yp); put(true, d.asc_y, h.att_yv); }
        } else {
            q.frame_f += (int64_t)d.nx * d.ny;
        }
        if (!d.rigid) q.cells += (int64_t)d.nx * d.ny;
    }
    q.set_f = (size_t)std::max<long long>(off, 32);
    q.fixed_f = (size_t)std::max<long long>(foff, 32);
    q.p0_f = (size_t)std::max<long long>(poff, 32);
    q.aux_f = (size_t)q.n_steps * sc.receivers.size() + 32;
    q.lengths.clear();
    for (const StripRun& r : sc.runs) {
        const int L = Kernel::run_length(sc, r);
        if (std::find(q.lengths.begin(), q.lengths.end(), L) == q.lengths.end()) q.lengths.push_back(L);
    }
    std::sort(q.lengths.begin(), q.lengths.end());
}

struct Server {
    Kernel K;                                  // batched plan, tables, graphs; its fields are the arenas
    RangeAlloc aset, afixed, ap0, aaux;
    DevBuf<float> aux;                         // receiver rings
    DevBuf<int> scene_step;                    // steps taken per slot
    DevBuf<int> scene_limit;                   // steps requested per slot
    DevBuf<DevSrvReceiver> drec;
    DevBuf<int> dslots;
    std::vector<float> att;
    std::map<std::tuple<int, int, int, float, float, float>, int> att_off;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::vector<int> free_slots;
    std::map<int, const StageVariant*> var_cache;   // stage-kernel variant per strip length (tuned once)
    int forced = -1;
    int64_t budget = 0, next_id = 1, cell_steps = 0, n_done = 0, rebuilds = 0, peak_bytes = 0;
    bool dirty = false;
    // persistent form: the domain table and the job regions of one array as
    // arenas of entries, each scene's entries written once at admission and
    // zeroed at release.  Set 0 (one merged launch per stage): two regions,
    // transform length >= 1024 (taken first) and the rest with the copy jobs.
    // Set 1 (one persistent launch per strip length): a region per length, a
    // scene's copy jobs in the region of its shortest length.  Counts in
    // device memory: {set 0: region 0 top, region 1 top, region 1 base; PML
    // domains, PML blocks, receivers, slots; set 1: top of region r at 7 + r}.
    struct Region {
        int L = 0;                         // set 1: the region's length; set 0: 1024 (long) or 0 (the rest)
        const StageVariant* var = nullptr; // set 1: the configuration of the region's launch
        RangeAlloc a;
        size_t base = 0;                   // first entry in the job array
    };
    static constexpr int MAX_REGIONS = 16;
    bool pers_allowed = true, pers = false;
    int pset = 1;                          // configuration set of the persistent form
    RangeAlloc adom;
    std::vector<Region> regs;
    DevBuf<int> dcount;
    int counts[7 + MAX_REGIONS] = {};
    size_t filt_up = 0, tw_up = 0, win_up = 0;   // host-table entries already on the device
    int64_t captures = 0, updates = 0;

    int64_t bytes_in_use() const {
        return (int64_t)(3 * aset.used + afixed.used + ap0.used + aaux.used) * 4;
    }

    void create(int64_t budget_bytes, int max_scenes) {
        if (const char* e = std::getenv("PSTD_AUTOTUNE")) K.autotune = std::atoi(e) != 0;
        if (const char* e = std::getenv("PSTD_VARIANT")) { forced = std::atoi(e); K.autotune = false; }
        if (const char* e = std::getenv("PSTD_SERVE_PERSISTENT")) pers_allowed = std::atoi(e) != 0;
        if (const char* e = std::getenv("PSTD_SERVE_FORM")) pset = std::string(e) == "merged" ? 0 : 1;
        budget = budget_bytes;
        CK(cudaGetDevice(&K.device));
        CK(cudaDeviceGetAttribute(&K.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, K.device));
        CK(cudaStreamCreateWithFlags(&K.stream, cudaStreamNonBlocking));
        // budget split: three state sets 25 % each, p0 10 %, fixed 8 %, rings 7 %
        const size_t floats = (size_t)(budget_bytes / 4);
        const size_t S = floats / 100 * 25, P = floats / 100 * 10, F = floats / 100 * 8;
        const size_t X = floats - 3 * S - P - F;
        for (auto& s : K.sets) s.alloc(S);
        K.fixed.alloc(F);
        K.p0.alloc(P);
        aux.alloc(X);
        aset.init(S);
        afixed.init(F);
        ap0.init(P);
        aaux.init(X);
        K.first_step.alloc(max_scenes);
        scene_step.alloc(max_scenes);
        scene_limit.alloc(max_scenes);
        CK(cudaMemset(K.first_step.p, 0, max_scenes * sizeof(int)));
        CK(cudaMemset(scene_step.p, 0, max_scenes * sizeof(int)));
        CK(cudaMemset(scene_limit.p, 0, max_scenes * sizeof(int)));
        for (int i = max_scenes - 1; i >= 0; i--) free_slots.push_back(i);
        K.srv.on = true;
        K.srv.n_flags = max_scenes;
        K.srv.aux = aux.p;
        K.srv.scene_step = scene_step.p;
        K.srv.limit = scene_limit.p;
        K.cur = 0;
        dcount.alloc(7 + MAX_REGIONS);
        CK(cudaMemset(dcount.p, 0, (7 + MAX_REGIONS) * sizeof(int)));
    }

    int64_t submit(const pstd_config* cfg, int n_steps, int flags) {
        if (n_steps <= 0) throw SceneError(PSTD_ERR_INVALID, "n_steps must be positive");
        auto q = std::make_unique<Request>();
        q->scene.build(cfg);
        if (q->scene.spectral) throw SceneError(PSTD_ERR_UNSUPPORTED, "spectral receivers are not served");
        q->n_steps = n_steps;
        q->flags = flags;
        layout_scene(*q, att, att_off);
        if (aset.round(q->set_f) > aset.cap || afixed.round(q->fixed_f) > afixed.cap ||
            ap0.round(q->p0_f) > ap0.cap || aaux.round(q->aux_f) > aaux.cap)
            throw SceneError(PSTD_ERR_NO_MEMORY, "request needs " + std::to_string(q->bytes()) +
                                                     " bytes of device memory, more than the server's arenas hold (budget " +
                                                     std::to_string(budget) + " bytes)");
        for (const StripRun& r : q->scene.runs) {
            const int L = Kernel::run_length(q->scene, r);
            const StageVariant* vs;
            if (stage_variants(L, &vs) <= 0)
                throw SceneError(PSTD_ERR_UNSUPPORTED, "strip transform length " + std::to_string(L) +
                                                           " is outside the compiled range 32..8192");
        }
        q->id = next_id++;
        Request* r = q.get();
        reqs[r->id] = std::move(q);
        queue.push_back(r);
        return r->id;
    }

    // admit queued requests in arrival order while their ranges fit
    std::vector<Request*> admit() {
        std::vector<Request*> fresh;
        while (!queue.empty() && !free_slots.empty()) {
            Request* q = queue.front();
            size_t a, b, c, d;
            if (!aset.alloc(q->set_f, &a)) break;
            if (!afixed.alloc(q->fixed_f, &b)) { aset.release(a, q->set_f); break; }
            if (!ap0.alloc(q->p0_f, &c)) { aset.release(a, q->set_f); afixed.release(b, q->fixed_f); break; }
            if (!aaux.alloc(q->aux_f, &d)) {
                aset.release(a, q->set_f); afixed.release(b, q->fixed_f); ap0.release(c, q->p0_f);
                break;
            }
            q->set_off = a; q->fixed_off = b; q->p0_off = c; q->aux_off = d;
            q->slot = free_slots.back();
            free_slots.pop_back();
            q->state = PSTD_REQ_ACTIVE;
            queue.pop_front();
            active.push_back(q);
            fresh.push_back(q);
        }
        peak_bytes = std::max(peak_bytes, bytes_in_use());
        return fresh;
    }

    void release(Request* q) {
        aset.release(q->set_off, q->set_f);
        afixed.release(q->fixed_off, q->fixed_f);
        ap0.release(q->p0_off, q->p0_f);
        aaux.release(q->aux_off, q->aux_f);
        if (q->placed) unplace(q);
        free_slots.push_back(q->slot);
        q->slot = -1;
        active.erase(std::find(active.begin(), active.end(), q));
        dirty = true;
    }

    // The scene's domain-table entry k: field offsets in the arenas, the slot as scene
    DevDomain global_domain(const Request* q, size_t k) const {
        DevDomain h = q->local[k];
        const long long so = h.fixed ? (long long)q->fixed_off : (long long)q->set_off;
        h.o_px += so; h.o_py += so; h.o_vx += so; h.o_vy += so;
        h.o_p0 += (long long)q->p0_off;
        h.scene = q->slot;
        return h;
    }

    // PML list with block prefix sums, receivers and slots of the active
    // scenes (domain indices from `base`, the index of each scene's first domain)
    void small_tables(const std::vector<size_t>& base, std::vector<int>& pml, std::vector<int>& off,
                      std::vector<DevSrvReceiver>& rec, std::vector<int>& slots) const {
        off.assign(1, 0);
        for (size_t si = 0; si < active.size(); si++) {
            const Request* q = active[si];
            for (size_t k = 0; k < q->local.size(); k++) {
                const DevDomain& h = q->local[k];
                if (!h.pml) continue;
                pml.push_back((int)(base[si] + k));
                off.push_back(off.back() + (h.ny + 1) * ((h.nx + 1 + 127) >> 7));
            }
            const int nr = (int)q->scene.receivers.size();
            for (int r = 0; r < nr; r++) {
                const Receiver& R = q->scene.receivers[r];
                rec.push_back({(int)base[si] + R.dom, R.row, R.col, q->slot, (long long)q->aux_off, nr, r});
            }
            slots.push_back(q->slot);
        }
    }

    // ---------------------------------------------------------------- per-length form
    // batched plan of the active scenes: domain table, receivers, buckets,
    // jobs, tuned variants and the three step graphs, all built afresh
    void rebuild_per_length() {
        pers = false;
        for (Request* q : active) q->placed = false;
        K.dev_counts = nullptr;
        K.dev_regions.clear();
        K.merged = false;
        K.scenes.clear(); K.dom_base.clear(); K.rec_base.clear(); K.gdom.clear(); K.buckets.clear();
        std::vector<DevDomain> hd;
        std::vector<size_t> base;
        for (size_t si = 0; si < active.size(); si++) {
            Request* q = active[si];
            q->dom_off = hd.size();
            base.push_back(hd.size());
            K.dom_base.push_back((int)hd.size());
            K.rec_base.push_back(0);
            K.scenes.push_back(q->scene);
            for (size_t k = 0; k < q->local.size(); k++) {
                K.gdom.push_back({(int)si, (int)k});
                hd.push_back(global_domain(q, k));
            }
        }
        std::vector<int> pml, off, slots;
        std::vector<DevSrvReceiver> rec;
        small_tables(base, pml, off, rec, slots);
        K.hdoms = hd;
        K.ddoms.upload(hd);
        K.n_pml = (int)pml.size();
        K.dpml.upload(pml);
        K.pml_blocks = off.back();
        K.dpml_off.upload(off);
        K.n_rec = (int)rec.size();
        drec.upload(rec);
        dslots.upload(slots);
        K.datt.upload(att.empty() ? std::vector<float>{1.f} : att);
        K.srv.rec = drec.p;
        K.srv.slots = dslots.p;
        K.srv.n_slots = (int)slots.size();

        std::vector<int> Ls;
        for (auto& sc : K.scenes)
            for (const StripRun& r : sc.runs) {
                const int L = Kernel::run_length(sc, r);
                if (std::find(Ls.begin(), Ls.end(), L) == Ls.end()) Ls.push_back(L);
            }
        std::sort(Ls.begin(), Ls.end());
        std::vector<bool> tune;
        for (int L : Ls) {
            const StageVariant* vs;
            const int nv = stage_variants(L, &vs);
            Bucket b;
            b.L = L;
            int longest = 0;
            for (auto& sc : K.scenes)
                for (const StripRun& r : sc.runs)
                    if (Kernel::run_length(sc, r) == L) longest = std::max(longest, sc.doms[r.dom].len(r.axis));
            b.rc = (longest + 2 + 3) / 4 * 4;
            bool need = false;
            if (forced >= 0) {
                b.var = &vs[std::min(forced, fp32_variants(vs, nv) - 1)];
                b.choice = " pinned";
            } else if (var_cache.count(L)) {
                b.var = var_cache[L];
            } else {
                for (int i = 0; i < nv; i++) CK(vs[i].prepare());
                b.var = &vs[0];
                need = K.autotune;
            }
            if (b.var->smem_for(b.rc) > (size_t)K.smem_optin) b.var = &vs[0];   // staging of this form does not fit
            if (forced >= 0) CK(b.var->prepare());
            K.buckets.push_back(b);
            tune.push_back(need);
        }
        const bool any = std::find(tune.begin(), tune.end(), true) != tune.end();
        K.plan(any, &tune);
        for (size_t i = 0; i < K.buckets.size(); i++)
            if (tune[i] && forced < 0) var_cache[K.buckets[i].L] = K.buckets[i].var;
        while (K.side.size() < K.buckets.size()) {
            cudaStream_t s;
            CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            K.side.push_back(s);
        }
        K.capture_graphs();
        captures++;
    }

    // ---------------------------------------------------------------- persistent form
    // first capacity of a table: `c` entries (PSTD_SERVE_TABLE_DIVISOR=d > 1
    // starts the tables d times smaller, so that tests exercise their growth)
    static size_t first_cap(size_t c) {
        const char* e = std::getenv("PSTD_SERVE_TABLE_DIVISOR");   // (read at every setup: tests set it per server)
        const size_t d = e && std::atoi(e) > 1 ? (size_t)std::atoi(e) : (size_t)1;
        return std::max<size_t>(c / d, 1);
    }

    // contents of v into b on the server's stream; b is reallocated (twice
    // the size needed, at least min_cap) when v does not fit.  True when the
    // device address changed.
    template <class T>
    bool put(DevBuf<T>& b, const std::vector<T>& v, size_t min_cap) {
        bool moved = false;
        if (!b.p || b.n < v.size()) {
            b.alloc(std::max({2 * v.size(), min_cap, 2 * b.n}));
            moved = true;
        }
        // pageable source: the copy has taken the data when the call returns
        if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, K.stream));
        return moved;
    }

    // the configuration of length L in set `set` (nullptr: not compiled there)
    static const StageVariant* set_variant(int set, int L, int fam) {
        if (set == 0) return merged_supports(L) ? merged_variant(L, fam) : nullptr;
        return serve_variant(L);
    }

    // the persistent form can run the scene: every strip length has a configuration
    bool runs_persistent(const Request* q) const {
        for (int L : q->lengths)
            if (!set_variant(pset, L, K.merged_fam)) return false;
        return true;
    }

    // the strip jobs of one scene for configuration set pset (Kernel::make_jobs
    // on the scene alone: domain indices local to the scene), by length
    void build_jobs(Request* q) {
        if (q->jobs_set == pset) return;
        q->jobs.clear();
        std::vector<Scene> keep_s;
        std::vector<int> keep_b;
        std::vector<std::pair<int, int>> keep_g;
        std::swap(keep_s, K.scenes);
        std::swap(keep_b, K.dom_base);
        std::swap(keep_g, K.gdom);
        auto restore = [&]() {
            std::swap(keep_s, K.scenes);
            std::swap(keep_b, K.dom_base);
            std::swap(keep_g, K.gdom);
        };
        try {
            K.scenes.assign(1, q->scene);
            K.dom_base.assign(1, 0);
            for (size_t k = 0; k < q->local.size(); k++) K.gdom.push_back({0, (int)k});
            for (int L : q->lengths) q->jobs[L] = K.make_jobs(L, set_variant(pset, L, K.merged_fam), false);
            const int L0 = q->lengths.empty() ? 128 : q->lengths.front();
            q->jobs[0] = K.make_jobs(-1, set_variant(pset, L0, K.merged_fam), true);
        } catch (...) {
            restore();
            throw;
        }
        restore();
        q->jobs_set = pset;
    }

    // n entries of the domain table; when it is full it doubles (contents
    // kept).  True when the table moved.
    bool take_domains(size_t n, size_t* off) {
        if (adom.alloc(n, off)) return false;
        const size_t c = std::max(2 * adom.cap, adom.cap + n);
        DevBuf<DevDomain> nb;
        nb.alloc(c);
        if (adom.cap)
            CK(cudaMemcpyAsync(nb.p, K.ddoms.p, adom.cap * sizeof(DevDomain), cudaMemcpyDeviceToDevice, K.stream));
        CK(cudaStreamSynchronize(K.stream));   // before the old table is freed
        std::swap(K.ddoms.p, nb.p);
        std::swap(K.ddoms.n, nb.n);
        adom.grow(c);
        if (!adom.alloc(n, off)) throw SceneError(PSTD_ERR_NO_MEMORY, "domain table");
        return true;
    }

    // the job array laid out again with region capacities caps (regions keep
    // their entries and offsets; free entries stay zero)
    void relayout(const std::vector<size_t>& caps) {
        size_t total = 0;
        std::vector<size_t> base;
        for (size_t c : caps) {
            base.push_back(total);
            total += c;
        }
        DevBuf<DevJob> nb;
        nb.alloc(std::max<size_t>(total, 1));
        CK(cudaMemsetAsync(nb.p, 0, nb.n * sizeof(DevJob), K.stream));
        for (size_t r = 0; r < regs.size(); r++)
            if (regs[r].a.cap)
                CK(cudaMemcpyAsync(nb.p + base[r], K.djobs_all.p + regs[r].base, regs[r].a.cap * sizeof(DevJob),
                                   cudaMemcpyDeviceToDevice, K.stream));
        CK(cudaStreamSynchronize(K.stream));   // before the old array is freed
        std::swap(K.djobs_all.p, nb.p);
        std::swap(K.djobs_all.n, nb.n);
        for (size_t r = 0; r < regs.size(); r++) {
            regs[r].base = base[r];
            regs[r].a.grow(caps[r]);
        }
    }

    // the region of jobs of length key (0: copy jobs) of a scene; set 1 adds
    // a region for a new length (the array is laid out again: *moved)
    int region_of(const Request* q, int key, bool* moved) {
        if (pset == 0) return key >= 1024 ? 0 : 1;
        const int L = key ? key : q->lengths.front();
        for (size_t r = 0; r < regs.size(); r++)
            if (regs[r].L == L) return (int)r;
        if ((int)regs.size() >= MAX_REGIONS) throw SceneError(PSTD_ERR_UNSUPPORTED, "too many strip lengths");
        Region g;
        g.L = L;
        g.var = serve_variant(L);
        CK(g.var->prepare_dev());
        g.a.init(0, 1);
        regs.push_back(g);
        std::vector<size_t> caps;
        for (const Region& x : regs) caps.push_back(x.a.cap ? x.a.cap : first_cap(1024));
        relayout(caps);
        *moved = true;
        return (int)regs.size() - 1;
    }

    // n entries of region r; a full region doubles (the array is laid out
    // again).  True when the array moved.
    bool take_jobs(int r, size_t n, size_t* off) {
        *off = 0;
        if (n == 0) return false;
        if (regs[r].a.alloc(n, off)) return false;
        std::vector<size_t> caps;
        for (const Region& x : regs) caps.push_back(x.a.cap);
        caps[r] = std::max(2 * caps[r], caps[r] + n);
        relayout(caps);
        if (!regs[r].a.alloc(n, off)) throw SceneError(PSTD_ERR_NO_MEMORY, "job table");
        return true;
    }

    // write a scene's domain entries and jobs into its table ranges
    bool place(Request* q) {
        build_jobs(q);
        bool moved = take_domains(q->local.size(), &q->dom_off);
        q->job_ranges.clear();
        for (const auto& kv : q->jobs) {
            const int r = region_of(q, kv.first, &moved);
            size_t off = 0;
            moved |= take_jobs(r, kv.second.size(), &off);
            q->job_ranges.push_back({r, off});
        }
        std::vector<DevDomain> hd;
        for (size_t k = 0; k < q->local.size(); k++) hd.push_back(global_domain(q, k));
        CK(cudaMemcpyAsync(K.ddoms.p + q->dom_off, hd.data(), hd.size() * sizeof(DevDomain), cudaMemcpyHostToDevice,
                           K.stream));
        const int o = (int)q->dom_off;
        size_t i = 0;
        for (const auto& kv : q->jobs) {   // (the array has its final layout now)
            const auto [r, off] = q->job_ranges[i++];
            if (kv.second.empty()) continue;
            std::vector<DevJob> g = kv.second;
            for (DevJob& j : g) {
                j.dom += o;
                if (j.d1 >= 0) j.d1 += o;
                if (j.d2 >= 0) j.d2 += o;
            }
            CK(cudaMemcpyAsync(K.djobs_all.p + regs[r].base + off, g.data(), g.size() * sizeof(DevJob),
                               cudaMemcpyHostToDevice, K.stream));
        }
        q->placed = true;
        return moved;
    }

    // zero a scene's jobs (skipped from the next launch on) and free its ranges
    void unplace(Request* q) {
        size_t i = 0;
        for (const auto& kv : q->jobs) {
            const auto [r, off] = q->job_ranges[i++];
            if (kv.second.empty()) continue;
            CK(cudaMemsetAsync(K.djobs_all.p + regs[r].base + off, 0, kv.second.size() * sizeof(DevJob), K.stream));
            regs[r].a.release(off, kv.second.size());
        }
        adom.release(q->dom_off, q->local.size());
        q->placed = false;
    }

    // persistent form of a membership change: new scenes placed, the small
    // tables and counts rewritten in place; the graphs are captured again only
    // when a table moved (or the form changed)
    void rebuild_persistent() {
        bool moved = false;
        if (!pers) {
            K.scenes.clear(); K.dom_base.clear(); K.rec_base.clear(); K.gdom.clear(); K.buckets.clear();
            adom.init(first_cap(4096), 1);
            K.ddoms.alloc(adom.cap);
            regs.clear();
            K.djobs_all.alloc(1);
            if (pset == 0) {
                regs.resize(2);
                regs[0].L = 1024;
                regs[0].a.init(0, 1);
                regs[1].a.init(0, 1);
                relayout({first_cap(1 << 15), first_cap(1 << 16)});
                CK(prepare_stage_all(K.merged_fam));
            }
            for (Request* q : active) q->placed = false;
            if (K.counters.n < 6 * MAX_REGIONS) K.counters.alloc(6 * MAX_REGIONS);
            filt_up = tw_up = win_up = 0;
            moved = true;
        }
        for (Request* q : active)
            if (!q->placed) moved |= place(q);
        std::vector<size_t> base;
        for (Request* q : active) base.push_back(q->dom_off);
        std::vector<int> pml, off, slots;
        std::vector<DevSrvReceiver> rec;
        small_tables(base, pml, off, rec, slots);
        moved |= put(K.dpml, pml, 4096);
        moved |= put(K.dpml_off, off, 4097);
        moved |= put(drec, rec, 1 << 14);
        moved |= put(dslots, slots, (size_t)K.srv.n_flags);
        std::vector<Kernel::DevRegion> launches;
        for (size_t r = 0; r < regs.size() && pset == 1; r++)
            launches.push_back({regs[r].var, regs[r].base, 7 + (int)r, K.twiddles_of(regs[r].var)});
        if (K.filt.size() != filt_up) { moved |= put(K.dfilt, K.filt, 1 << 15); filt_up = K.filt.size(); }
        if (K.tw.size() != tw_up) { moved |= put(K.dtw, K.tw, 1 << 15); tw_up = K.tw.size(); }
        if (K.win.size() != win_up) { moved |= put(K.dwin, K.win, 1 << 13); win_up = K.win.size(); }
        moved |= put(K.datt, att.empty() ? std::vector<float>{1.f} : att, 1 << 13);
        std::fill(std::begin(counts), std::end(counts), 0);
        if (pset == 0) {
            counts[0] = (int)regs[0].a.top();
            counts[1] = (int)regs[1].a.top();
            counts[2] = (int)regs[1].base;
        }
        counts[3] = (int)pml.size();
        counts[4] = off.back();
        counts[5] = (int)rec.size();
        counts[6] = (int)slots.size();
        for (size_t r = 0; r < regs.size(); r++) counts[7 + r] = (int)regs[r].a.top();
        CK(cudaMemcpyAsync(dcount.p, counts, sizeof counts, cudaMemcpyHostToDevice, K.stream));
        K.n_all = pset == 0 ? counts[0] + counts[1] : 0;
        K.n_pml = counts[3];
        K.pml_blocks = counts[4];
        K.n_rec = counts[5];
        K.sep.clear();
        K.merged = true;
        K.dev_counts = dcount.p;
        K.dev_regions = launches;
        K.srv.rec = drec.p;
        K.srv.slots = dslots.p;
        K.srv.n_slots = counts[6];
        while (K.side.size() < regs.size() + 1) {
            cudaStream_t st;
            CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            K.side.push_back(st);
        }
        if (moved) {
            K.capture_graphs();
            captures++;
        } else {
            updates++;
        }
        pers = true;
    }

    // initial condition of newly admitted scenes in the current state set
    void init(const std::vector<Request*>& fresh) {
        for (Request* q : fresh) {
            CK(cudaMemsetAsync(K.sets[K.cur].p + q->set_off, 0, q->set_f * sizeof(float), K.stream));
            CK(cudaMemsetAsync(K.fixed.p + q->fixed_off, 0, q->fixed_f * sizeof(float), K.stream));
            CK(cudaMemsetAsync(K.p0.p + q->p0_off, 0, q->p0_f * sizeof(float), K.stream));
            CK(cudaMemsetAsync(scene_step.p + q->slot, 0, sizeof(int), K.stream));
            CK(cudaMemcpyAsync(scene_limit.p + q->slot, &q->n_steps, sizeof(int), cudaMemcpyHostToDevice, K.stream));
            static const int one = 1;
            CK(cudaMemcpyAsync(K.first_step.p + q->slot, &one, sizeof(int), cudaMemcpyHostToDevice, K.stream));
            const Scene& sc = q->scene;
            if (!sc.speakers.empty()) {
                std::vector<int> x0, y0;
                for (auto& d : sc.doms) { x0.push_back(d.x0); y0.push_back(d.y0); }
                std::vector<DevSpeaker> spk;
                for (auto& s : sc.speakers) spk.push_back({s.x, s.y});
                DevBuf<int> dx0, dy0;
                DevBuf<DevSpeaker> dspk;
                dx0.upload(x0);
                dy0.upload(y0);
                dspk.upload(spk);
                CK(launch_speakers(K.ddoms.p + q->dom_off, dx0.p, dy0.p, (int)sc.doms.size(), dspk.p, (int)spk.size(),
                                   sc.s.dx, sc.s.band_width, K.sets[K.cur].p, K.fixed.p, K.p0.p, K.stream));
                CK(cudaStreamSynchronize(K.stream));
            }
        }
        CK(cudaStreamSynchronize(K.stream));
    }

    // p0 = px + py of every non-PML domain of a scene, scene order, from the
    // state set of its last step
    void final_frame(Request* q) {
        q->frame.assign(q->frame_f, 0.f);
        size_t at = 0;
        std::vector<float> a, b;
        for (size_t k = 0; k < q->local.size(); k++) {
            const DevDomain& d = q->local[k];
            if (d.pml) continue;
            const float* base = d.fixed ? K.fixed.p + q->fixed_off : K.sets[q->final_set].p + q->set_off;
            const size_t n = (size_t)d.nx * d.ny;
            a.resize(n);
            b.resize(n);
            CK(cudaMemcpy2D(a.data(), d.nx * sizeof(float), base + d.o_px, d.pitch_p * sizeof(float), d.nx * sizeof(float),
                            d.ny, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy2D(b.data(), d.nx * sizeof(float), base + d.o_py, d.pitch_p * sizeof(float), d.nx * sizeof(float),
                            d.ny, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < n; i++) q->frame[at + i] = a[i] + b[i];
            at += n;
        }
    }

    // info[4] = {active, queued, finished in this tick, steps advanced}.  The
    // per-length form advances every scene by the same number of steps, no
    // further than the scene closest to completion; the persistent form runs
    // up to max_steps and scenes that reach their step count stop on the
    // device (their jobs, PML pass and receivers are skipped) until the tick ends.
    void tick(int max_steps, int32_t* info) {
        std::vector<Request*> fresh = admit();
        if ((dirty || !fresh.empty()) && !active.empty()) {
            bool merge = pers_allowed && forced < 0;
            for (const Request* q : active) merge = merge && runs_persistent(q);
            if (merge) rebuild_persistent();
            else rebuild_per_length();
            rebuilds++;
        }
        dirty = false;
        init(fresh);
        int T = 0, finished = 0;
        if (!active.empty()) {
            int most = 0, least = INT32_MAX;
            for (const Request* q : active) {
                most = std::max(most, q->n_steps - q->steps_done);
                least = std::min(least, q->n_steps - q->steps_done);
            }
            T = std::max(1, std::min(max_steps, pers ? most : least));
            const int c0 = K.cur;
            for (int t = 0; t < T; t++) K.step(K.stream);
            CK(cudaStreamSynchronize(K.stream));
            std::vector<Request*> done;
            for (Request* q : active) {
                const int k = std::min(T, q->n_steps - q->steps_done);
                q->steps_done += k;
                q->final_set = (c0 + 2 * k) % 3;
                cell_steps += q->cells * k;
                if (q->steps_done >= q->n_steps) done.push_back(q);
            }
            for (Request* q : done) {
                const size_t nr = q->scene.receivers.size();
                q->receivers.assign((size_t)q->n_steps * nr, 0.f);
                if (nr)
                    CK(cudaMemcpy(q->receivers.data(), aux.p + q->aux_off, q->receivers.size() * sizeof(float),
                                  cudaMemcpyDeviceToHost));
                if (q->flags & PSTD_REQ_FINAL_FRAME) final_frame(q);
                q->state = PSTD_REQ_DONE;
                release(q);
                n_done++;
                finished++;
            }
        }
        if (info) {
            info[0] = (int32_t)active.size();
            info[1] = (int32_t)queue.size();
            info[2] = finished;
            info[3] = T;
        }
    }

    void cancel(Request* q) {
        if (q->state == PSTD_REQ_QUEUED) {
            queue.erase(std::find(queue.begin(), queue.end(), q));
        } else if (q->state == PSTD_REQ_ACTIVE) {
            release(q);
        }
        q->state = PSTD_REQ_CANCELLED;
    }
};

}  // namespace pstd

using namespace pstd;

struct pstd_server {
    std::unique_ptr<Server> s;
};

#define SRV_GUARD(...)                                                          \
    try {                                                                       \
        __VA_ARGS__                                                             \
    } catch (SceneError & e) {                                                  \
        return set_error(e.code, e.what());                                     \
    } catch (CudaError & e) {                                                   \
        return set_error(PSTD_ERR_CUDA, e.what());                              \
    } catch (std::bad_alloc&) {                                                 \
        return set_error(PSTD_ERR_NO_MEMORY, "allocation failed");              \
    } catch (std::exception & e) {                                              \
        return set_error(PSTD_ERR_INVALID, e.what());                           \
    }

#define NEED_SRV(h) \
    if (!(h) || !(h)->s) return set_error(PSTD_ERR_NOT_CONFIGURED, "server handle is not configured");

static Request* find_req(Server* s, int64_t id) {
    auto it = s->reqs.find(id);
    return it == s->reqs.end() ? nullptr : it->second.get();
}

extern "C" {

int pstd_server_create(int64_t hbm_budget_bytes, int32_t max_scenes, const pstd_callbacks* log_cb, pstd_server** out) {
    if (!out) return set_error(PSTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (hbm_budget_bytes < (1 << 20) || max_scenes <= 0)
        return set_error(PSTD_ERR_INVALID, "budget must be at least 1 MiB and max_scenes positive");
    SRV_GUARD({
        auto h = std::make_unique<pstd_server>();
        h->s = std::make_unique<Server>();
        if (log_cb) { h->s->K.logcb = *log_cb; h->s->K.have_logcb = true; }
        h->s->create(hbm_budget_bytes, max_scenes);
        *out = h.release();
        return PSTD_OK;
    })
}

void pstd_server_destroy(pstd_server* h) {
    if (!h) return;
    try {
        if (h->s && h->s->K.stream) cudaStreamSynchronize(h->s->K.stream);
        delete h;
    } catch (...) {
    }
}

int pstd_server_submit(pstd_server* h, const pstd_config* config, int32_t n_steps, int32_t flags, int64_t* request_id) {
    NEED_SRV(h);
    if (!config || !request_id) return set_error(PSTD_ERR_INVALID, "config or request_id is NULL");
    SRV_GUARD({
        *request_id = h->s->submit(config, n_steps, flags);
        return PSTD_OK;
    })
}

int pstd_server_tick(pstd_server* h, int32_t max_steps, int32_t* info) {
    NEED_SRV(h);
    if (max_steps <= 0) return set_error(PSTD_ERR_INVALID, "max_steps must be positive");
    SRV_GUARD({
        h->s->tick(max_steps, info);
        return PSTD_OK;
    })
}

int pstd_server_poll(pstd_server* h, int64_t request_id, int32_t* state, int32_t* steps_done, int64_t* sizes) {
    NEED_SRV(h);
    Request* q = find_req(h->s.get(), request_id);
    if (!q) return set_error(PSTD_ERR_INVALID, "unknown request id");
    if (state) *state = q->state;
    if (steps_done) *steps_done = q->steps_done;
    if (sizes) {
        sizes[0] = (int64_t)q->n_steps * (int64_t)q->scene.receivers.size();
        sizes[1] = (q->flags & PSTD_REQ_FINAL_FRAME) ? q->frame_f : 0;
    }
    return PSTD_OK;
}

int pstd_server_result(pstd_server* h, int64_t request_id, float* receivers, int64_t n_receivers, float* frame,
                       int64_t n_frame) {
    NEED_SRV(h);
    Server* s = h->s.get();
    Request* q = find_req(s, request_id);
    if (!q) return set_error(PSTD_ERR_INVALID, "unknown request id");
    if (q->state != PSTD_REQ_DONE) return set_error(PSTD_ERR_INVALID, "request has not finished");
    if ((int64_t)q->receivers.size() != n_receivers || (int64_t)q->frame.size() != n_frame)
        return set_error(PSTD_ERR_INVALID, "result sizes do not match pstd_server_poll's");
    if (n_receivers) std::memcpy(receivers, q->receivers.data(), n_receivers * sizeof(float));
    if (n_frame) std::memcpy(frame, q->frame.data(), n_frame * sizeof(float));
    s->reqs.erase(request_id);
    return PSTD_OK;
}

int pstd_server_cancel(pstd_server* h, int64_t request_id) {
    NEED_SRV(h);
    Server* s = h->s.get();
    Request* q = find_req(s, request_id);
    if (!q) return set_error(PSTD_ERR_INVALID, "unknown request id");
    if (q->state == PSTD_REQ_DONE || q->state == PSTD_REQ_CANCELLED) return PSTD_OK;
    s->cancel(q);
    return PSTD_OK;
}

int pstd_server_stats(pstd_server* h, int64_t* stats) {
    NEED_SRV(h);
    Server* s = h->s.get();
    stats[0] = s->budget;
    stats[1] = s->bytes_in_use();
    stats[2] = s->peak_bytes;
    stats[3] = s->cell_steps;
    stats[4] = s->n_done;
    stats[5] = s->rebuilds;
    stats[6] = (int64_t)s->active.size();
    stats[7] = (int64_t)s->queue.size();
    return PSTD_OK;
}

int pstd_server_launch_stats(pstd_server* h, int64_t* out) {
    NEED_SRV(h);
    if (!out) return set_error(PSTD_ERR_INVALID, "out is NULL");
    Server* s = h->s.get();
    out[0] = s->captures;
    out[1] = s->updates;
    out[2] = s->pers ? 1 : 0;
    out[3] = s->active.empty() ? 0 : s->K.launches_per_step();
    return PSTD_OK;
}

}  // extern "C"
