// server.cu -- the serving loop: continuous batching of scene solves on one
// GPU (include/pstd_gb300.h, pstd_server_*).
//
// Requests (a scene and a step count) are built on the host at submit time,
// queue, and are admitted -- in arrival order -- when their fields fit the
// device arenas (admission by HBM footprint).  All admitted scenes form one
// batch: every RK stage launches the stage kernel once per strip-length
// bucket over the strips of all active scenes (the batched plan of
// pstd_create_batch), captured as CUDA graphs per membership.  A tick
// advances every active scene by the same number of steps, no further than
// the scene closest to completion; then finished scenes hand their receiver
// series (and optionally the last frame) to the host and free their arena
// ranges, and waiting requests are admitted into the freed space.  Scenes that
// join later run in the same launches as the ones already running: their work
// overlaps on the device.
//
// Device memory is reserved once (the budget): three state-set arenas of equal
// layout (a scene has the same offset in all three), the fixed-buffer arena of
// rigid domains, the p0 arena and an auxiliary arena for receiver rings.  The
// results of a scene do not depend on the other scenes of the batch: every
// strip job reads and writes only its own scene's fields.
#include <cuda_runtime.h>

#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pstd_gb300.h"
#include "kernel_state.hpp"

namespace pstd {

// first-fit allocator of float ranges (multiples of 64 floats = 256 bytes)
struct RangeAlloc {
    size_t cap = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_;   // offset -> length

    static size_t round(size_t n) { return (std::max<size_t>(n, 1) + 63) / 64 * 64; }
    void init(size_t c) {
        cap = c / 64 * 64;
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

    int64_t bytes() const { return (int64_t)(3 * set_f + fixed_f + p0_f + aux_f) * 4; }
};

// Field layout of one scene relative to its own ranges (the layout pstd_create
// uses, device.cuh); attenuation profiles are appended to the shared table.
static void layout_scene(Request& q, std::vector<float>& att, std::map<std::tuple<int, int, int, float, float, float>, int>& att_off) {
    const Scene& sc = q.scene;
    auto round32 = [](long long v) { return (v + 31) / 32 * 32; };
    long long off = 0, foff = 0, poff = 0;
    q.local.assign(sc.doms.size(), DevDomain{});
    q.cells = 0;
    q.frame_f = 0;
    for (size_t k = 0; k < sc.doms.size(); k++) {
        const Domain& d = sc.doms[k];
        DevDomain& h = q.local[k];
        std::memset(&h, 0, sizeof h);
        h.nx = d.nx; h.ny = d.ny;
        h.pitch_p = (int)round32(d.nx);
        h.pitch_vx = (int)round32(d.nx + 1);
        h.pitch_vy = (int)round32(d.nx);
        h.fixed = d.rigid;
        long long& o = d.rigid ? foff : off;
        h.o_px = o; o = round32(o + (long long)h.pitch_p * d.ny);
        h.o_py = o; o = round32(o + (long long)h.pitch_p * d.ny);
        h.o_vx = o; o = round32(o + (long long)h.pitch_vx * d.ny);
        h.o_vy = o; o = round32(o + (long long)h.pitch_vy * (d.ny + 1));
        h.o_p0 = poff; poff = round32(poff + (long long)h.pitch_p * d.ny);
        h.rho = d.rho;
        h.c2 = sc.s.c1 * sc.s.c1;
        const float dt = sc.s.dt();
        for (int i = 0; i < 6; i++) h.cdt[i] = dt * sc.s.rk[i];
        h.pml = d.pml;
        h.att_xp = h.att_xv = h.att_yp = h.att_yv = -1;
        if (d.pml) {
            // profiles depend on (PML cells, velocity, ascending, ampMax, dt, rho): shared across requests
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
}

struct Server {
    Kernel K;                                  // batched plan, tables, graphs; its fields are the arenas
    RangeAlloc aset, afixed, ap0, aaux;
    DevBuf<float> aux;                         // receiver rings
    DevBuf<int> scene_step;                    // steps taken per slot
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

    int64_t bytes_in_use() const {
        return (int64_t)(3 * aset.used + afixed.used + ap0.used + aaux.used) * 4;
    }

    void create(int64_t budget_bytes, int max_scenes) {
        if (const char* e = std::getenv("PSTD_AUTOTUNE")) K.autotune = std::atoi(e) != 0;
        if (const char* e = std::getenv("PSTD_VARIANT")) { forced = std::atoi(e); K.autotune = false; }
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
        CK(cudaMemset(K.first_step.p, 0, max_scenes * sizeof(int)));
        CK(cudaMemset(scene_step.p, 0, max_scenes * sizeof(int)));
        for (int i = max_scenes - 1; i >= 0; i--) free_slots.push_back(i);
        K.srv.on = true;
        K.srv.n_flags = max_scenes;
        K.srv.aux = aux.p;
        K.srv.scene_step = scene_step.p;
        K.cur = 0;
    }

    int64_t submit(const pstd_config* cfg, int n_steps, int flags) {
        if (n_steps <= 0) throw SceneError(PSTD_ERR_INVALID, "n_steps must be positive");
        auto q = std::make_unique<Request>();
        q->scene.build(cfg);
        q->n_steps = n_steps;
        q->flags = flags;
        layout_scene(*q, att, att_off);
        if (RangeAlloc::round(q->set_f) > aset.cap || RangeAlloc::round(q->fixed_f) > afixed.cap ||
            RangeAlloc::round(q->p0_f) > ap0.cap || RangeAlloc::round(q->aux_f) > aaux.cap)
            throw SceneError(PSTD_ERR_NO_MEMORY, "request needs " + std::to_string(q->bytes()) +
                                                     " bytes of device memory, more than the server's arenas hold (budget " +
                                                     std::to_string(budget) + " bytes)");
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
        free_slots.push_back(q->slot);
        q->slot = -1;
        active.erase(std::find(active.begin(), active.end(), q));
        dirty = true;
    }

    // batched plan of the active scenes: domain table, receivers, buckets,
    // jobs and the three step graphs
    void rebuild() {
        K.scenes.clear(); K.dom_base.clear(); K.rec_base.clear(); K.gdom.clear(); K.buckets.clear();
        std::vector<DevDomain> hd;
        std::vector<int> pml, slots;
        std::vector<DevSrvReceiver> rec;
        for (size_t si = 0; si < active.size(); si++) {
            const Request* q = active[si];
            K.dom_base.push_back((int)hd.size());
            K.rec_base.push_back((int)rec.size());
            K.scenes.push_back(q->scene);
            const int base = (int)hd.size();
            for (size_t k = 0; k < q->local.size(); k++) {
                K.gdom.push_back({(int)si, (int)k});
                DevDomain h = q->local[k];
                const long long so = h.fixed ? (long long)q->fixed_off : (long long)q->set_off;
                h.o_px += so; h.o_py += so; h.o_vx += so; h.o_vy += so;
                h.o_p0 += (long long)q->p0_off;
                h.scene = q->slot;
                if (h.pml) pml.push_back((int)hd.size());
                hd.push_back(h);
            }
            const int nr = (int)q->scene.receivers.size();
            for (int r = 0; r < nr; r++) {
                const Receiver& R = q->scene.receivers[r];
                rec.push_back({base + R.dom, R.row, R.col, q->slot, (long long)q->aux_off, nr, r});
            }
            slots.push_back(q->slot);
        }
        K.hdoms = hd;
        K.ddoms.upload(hd);
        K.n_pml = (int)pml.size();
        K.dpml.upload(pml);
        K.set_pml_blocks(pml);
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
            if (nv <= 0)
                throw SceneError(PSTD_ERR_UNSUPPORTED, "strip transform length " + std::to_string(L) +
                                                           " is outside the compiled range 32..8192");
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
        rebuilds++;
    }

    // initial condition of newly admitted scenes in the current state set
    void init(const std::vector<Request*>& fresh) {
        for (Request* q : fresh) {
            const int si = (int)(std::find(active.begin(), active.end(), q) - active.begin());
            const int base = K.dom_base[si];
            CK(cudaMemsetAsync(K.sets[K.cur].p + q->set_off, 0, q->set_f * sizeof(float), K.stream));
            CK(cudaMemsetAsync(K.fixed.p + q->fixed_off, 0, q->fixed_f * sizeof(float), K.stream));
            CK(cudaMemsetAsync(K.p0.p + q->p0_off, 0, q->p0_f * sizeof(float), K.stream));
            CK(cudaMemsetAsync(scene_step.p + q->slot, 0, sizeof(int), K.stream));
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
                CK(launch_speakers(K.ddoms.p + base, dx0.p, dy0.p, (int)sc.doms.size(), dspk.p, (int)spk.size(), sc.s.dx,
                                   sc.s.band_width, K.sets[K.cur].p, K.fixed.p, K.p0.p, K.stream));
                CK(cudaStreamSynchronize(K.stream));
            }
        }
        CK(cudaStreamSynchronize(K.stream));
    }

    // p0 = px + py of every non-PML domain of a scene, scene order
    void final_frame(Request* q) {
        q->frame.assign(q->frame_f, 0.f);
        size_t at = 0;
        std::vector<float> a, b;
        for (size_t k = 0; k < q->local.size(); k++) {
            const DevDomain& d = q->local[k];
            if (d.pml) continue;
            const float* base = d.fixed ? K.fixed.p + q->fixed_off : K.sets[K.cur].p + q->set_off;
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

    // info[4] = {active, queued, finished in this tick, steps advanced}
    void tick(int max_steps, int32_t* info) {
        std::vector<Request*> fresh = admit();
        if ((dirty || !fresh.empty()) && !active.empty()) rebuild();
        dirty = false;
        init(fresh);
        int T = 0, finished = 0;
        if (!active.empty()) {
            T = std::max(1, max_steps);
            for (Request* q : active) T = std::min(T, q->n_steps - q->steps_done);
            for (int t = 0; t < T; t++) K.step(K.stream);
            CK(cudaStreamSynchronize(K.stream));
            std::vector<Request*> done;
            for (Request* q : active) {
                q->steps_done += T;
                cell_steps += q->cells * T;
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

}  // extern "C"
