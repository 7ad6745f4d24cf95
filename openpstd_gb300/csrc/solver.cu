// solver.cu -- host runtime of the GB300 PSTD solve and the C ABI of
// include/pstd_gb300.h.
//
// pstd_create builds the scene on the host (scene.cpp), the FP64 tables
// (window, derivative filters, twiddles, PML profiles), the device field
// layout (device.cuh) and the strip-job plan, then uploads everything once.
// A time step (kernel/Solver.cpp:71-117) is six RK stages; each stage is one
// launch of the stage kernel per strip-length bucket, all buckets running
// concurrently (they read only the previous stage); then one PML kernel and
// one receiver gather.  The three phases of the state-set rotation are
// captured as three CUDA graphs.  For every bucket the stage-kernel variant
// (strips per CTA, threads, radix plan) is picked by timing each compiled
// variant on the scene's own jobs at create time.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/pstd_gb300.h"
#include "kernel_state.hpp"
#include "launch.hpp"
#include "scene.hpp"

namespace pstd {

static thread_local std::string g_error;

int set_error(int code, const std::string& message) {
    g_error = message;
    return code;
}


// save_nth > 0 overrides the scene's SaveNth; sub > 1 subsamples every frame
// on the device (every sub-th row and column) before it is copied out
static int run_frames(Kernel* k, const pstd_callbacks* cb, int save_nth = 0, int sub = 1) {
    if (k->scenes.size() != 1) throw SceneError(PSTD_ERR_INVALID, "run() delivers frames of a single scene; advance batches");
    const Scene& sc = k->scenes[0];
    const int nframes = k->framecount;
    const int save = save_nth > 0 ? save_nth : std::max(1, sc.s.save_nth);
    sub = std::max(1, sub);
    std::vector<long long> foff(k->frame_doms.size());
    std::vector<size_t> fn(k->frame_doms.size());
    size_t frame_floats = 0;
    for (size_t i = 0; i < k->frame_doms.size(); i++) {
        const DevDomain& d = k->hdoms[k->frame_doms[i]];
        foff[i] = (long long)frame_floats;
        fn[i] = (size_t)((d.nx + sub - 1) / sub) * (size_t)((d.ny + sub - 1) / sub);
        frame_floats += fn[i];
    }
    DevBuf<long long> dsub_off;
    if (sub > 1) dsub_off.upload(foff);
    const long long* doff = sub > 1 ? dsub_off.p : k->dframe_off.p;
    // Frames in flight.  A frame (and the step's receiver row) is formed on
    // the compute stream into its own device slot and copied to pinned host
    // memory on a copy stream, so the next steps do not queue behind the
    // copy.  A slot is refilled only after the host has delivered its
    // previous frame (the loop below waits for that), so neither the device
    // nor the host slot is overwritten while a copy reads it.
    // Small frames get more slots (up to 8, within 64 MiB) so that the
    // device runs further ahead of a host whose callbacks take uneven time.
    const size_t slot = frame_floats + (size_t)std::max(k->n_rec, 1);
    const size_t slot_bytes = (frame_floats + (size_t)k->n_rec) * sizeof(float);
    const int K = Kernel::run_slot_count(slot);
    k->reserve_run_slots(slot * K);   // (made at create for the common frame size: nothing to do then)
    PinnedBuf& stage = k->run_stage;
    DevBuf<float>& dslots = k->run_slots;
    struct Sync {   // events and the copy stream, released on every exit
        std::vector<cudaEvent_t> ready, done;
        cudaStream_t copy = nullptr;
        ~Sync() {
            if (copy) cudaStreamSynchronize(copy), cudaStreamDestroy(copy);
            for (auto e : ready) cudaEventDestroy(e);
            for (auto e : done) cudaEventDestroy(e);
        }
    } sy;
    for (int i = 0; i < K; i++) {
        cudaEvent_t a, b;
        CK(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
        sy.ready.push_back(a);
        CK(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
        sy.done.push_back(b);
    }
    CK(cudaStreamCreateWithFlags(&sy.copy, cudaStreamNonBlocking));
    auto& ev = sy.done;
    // per frame, the caller's destination of each domain's frame (nullptr: the staging slot)
    struct Pending { int frame, slot; std::vector<float*> dst; };
    std::deque<Pending> q;
    int status = PSTD_OK;
    auto log = [&](int lvl, const std::string& m) { if (cb && cb->log) cb->log(cb->user, lvl, m.c_str()); };
    auto deliver = [&](const Pending& p) {
        CK(cudaEventSynchronize(ev[p.slot]));
        float* base = stage.p + slot * p.slot;
        for (size_t i = 0; i < k->frame_doms.size(); i++) {
            int d = k->frame_doms[i];
            const float* data = (i < p.dst.size() && p.dst[i]) ? p.dst[i] : base + foff[i];
            if (cb && cb->write_frame && status == PSTD_OK)
                if (cb->write_frame(cb->user, p.frame, sc.doms[d].id, data, (int64_t)fn[i]) != 0)
                    status = PSTD_ERR_CALLBACK;
        }
        for (int r = 0; r < k->n_rec; r++) {
            if (cb && cb->write_sample && status == PSTD_OK)
                if (cb->write_sample(cb->user, p.frame, sc.receivers[r].id, base + frame_floats + r, 1) != 0)
                    status = PSTD_ERR_CALLBACK;
        }
        log(PSTD_LOG_INFO, "Finished frame: " + std::to_string(p.frame));
    };
    // frames leave the queue in frame order: saved ones after their callbacks,
    // unsaved ones (SaveNth > 1) as soon as every earlier frame has left, so
    // "Finished frame" is logged in frame order (kernel/Solver.cpp:86-92)
    int inflight = 0;
    auto pop_front = [&]() {
        const Pending p = q.front();
        q.pop_front();
        if (p.slot >= 0) {
            deliver(p);
            inflight--;
        } else {
            log(PSTD_LOG_INFO, "Finished frame: " + std::to_string(p.frame));
        }
    };
    log(PSTD_LOG_DEBUG, "Number of render time: " + std::to_string(sc.s.calctime));
    log(PSTD_LOG_DEBUG, "Size of time step: " + std::to_string(sc.s.dt()));
    log(PSTD_LOG_INFO, "Starting simulation");
    int next_slot = 0;
    for (int f = 0; f < nframes && status == PSTD_OK; f++) {
        k->step(k->stream);
        if (f % save == 0) {
            int s = next_slot;
            next_slot = (next_slot + 1) % K;
            float* base = stage.p + slot * s;
            float* dbase = dslots.p + slot * s;
            const int row = (k->steps - 1) % k->ring_cap;
            CK(launch_frame(k->dframe_doms.p, doff, frame_floats ? (int)k->frame_doms.size() : 0, k->ddoms.p,
                            k->sets[k->cur].p, dbase, k->stream, sub, k->dring.p + (size_t)row * k->n_rec, k->n_rec,
                            dbase + frame_floats));
            CK(cudaEventRecord(sy.ready[s], k->stream));
            CK(cudaStreamWaitEvent(sy.copy, sy.ready[s], 0));
            std::vector<float*> dst;
            if (cb && cb->frame_buffer && cb->write_frame) {
                // the caller's own buffers: one copy per domain, the receiver row to the staging slot
                for (size_t i = 0; i < k->frame_doms.size(); i++) {
                    float* p = cb->frame_buffer(cb->user, f, sc.doms[k->frame_doms[i]].id, (int64_t)fn[i]);
                    dst.push_back(p);
                    float* to = p ? p : base + foff[i];
                    if (fn[i]) CK(cudaMemcpyAsync(to, dbase + foff[i], fn[i] * sizeof(float), cudaMemcpyDeviceToHost, sy.copy));
                }
                if (k->n_rec)
                    CK(cudaMemcpyAsync(base + frame_floats, dbase + frame_floats, (size_t)k->n_rec * sizeof(float),
                                       cudaMemcpyDeviceToHost, sy.copy));
            } else if (slot_bytes) {
                CK(cudaMemcpyAsync(base, dbase, slot_bytes, cudaMemcpyDeviceToHost, sy.copy));
            }
            CK(cudaEventRecord(ev[s], sy.copy));
            q.push_back({f, s, std::move(dst)});
            inflight++;
        } else {
            q.push_back({f, -1, {}});   // logged once every earlier frame is delivered
        }
        while (!q.empty() && q.front().slot < 0 && status == PSTD_OK) pop_front();
        while (inflight >= K && status == PSTD_OK) {
            pop_front();
            while (!q.empty() && q.front().slot < 0 && status == PSTD_OK) pop_front();
        }
    }
    while (!q.empty()) {
        if (status == PSTD_OK) pop_front();
        else q.pop_front();
    }
    CK(cudaStreamSynchronize(k->stream));
    CK(cudaStreamSynchronize(sy.copy));
    k->check_stage_error();
    if (status == PSTD_OK) log(PSTD_LOG_INFO, "Succesfully finished simulation");
    else g_error = "a callback asked to stop the run";
    return status;
}

}  // namespace pstd

using namespace pstd;

struct pstd_kernel {
    std::unique_ptr<Kernel> k;
};

static int fail(int code, const std::string& m) {
    g_error = m;
    return code;
}

#define GUARD(...)                                                              \
    try {                                                                       \
        __VA_ARGS__                                                             \
    } catch (SceneError & e) {                                                  \
        return fail(e.code, e.what());                                          \
    } catch (CudaError & e) {                                                   \
        return fail(PSTD_ERR_CUDA, e.what());                                   \
    } catch (std::bad_alloc&) {                                                 \
        return fail(PSTD_ERR_NO_MEMORY, "host allocation failed");              \
    } catch (std::exception & e) {                                              \
        return fail(PSTD_ERR_INVALID, e.what());                                \
    }

#define NEED(h)                                                                                  \
    if (!(h) || !(h)->k) return fail(PSTD_ERR_NOT_CONFIGURED, "kernel handle is not configured");
#define NEED_DEVICE(h)                                                                           \
    NEED(h);                                                                                     \
    if ((h)->k->host_only) return fail(PSTD_ERR_NOT_CONFIGURED, "handle holds a host-only scene");

extern "C" {

const char* pstd_last_error(void) { return g_error.c_str(); }
const char* pstd_version(void) { return "pstd_gb300 0.2.0 (sm_103a)"; }

int pstd_create(const pstd_config* config, const pstd_callbacks* log_cb, pstd_kernel** out) {
    if (!out) return fail(PSTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    GUARD({
        auto h = std::make_unique<pstd_kernel>();
        h->k = std::make_unique<Kernel>();
        if (log_cb) { h->k->logcb = *log_cb; h->k->have_logcb = true; }
        h->k->log(PSTD_LOG_DEBUG, "Initializing kernel");
        h->k->build(config, 1);
        h->k->log(PSTD_LOG_DEBUG, "Finished initializing kernel");
        *out = h.release();
        return PSTD_OK;
    })
}

int pstd_scene_build(const pstd_config* config, pstd_kernel** out) {
    if (!out) return fail(PSTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    GUARD({
        auto h = std::make_unique<pstd_kernel>();
        h->k = std::make_unique<Kernel>();
        h->k->build_scenes(config, 1);
        h->k->host_only = true;
        *out = h.release();
        return PSTD_OK;
    })
}

int pstd_create_batch(const pstd_config* configs, int32_t n, const pstd_callbacks* log_cb, pstd_kernel** out) {
    if (!out) return fail(PSTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!configs || n <= 0) return fail(PSTD_ERR_INVALID, "empty batch");
    GUARD({
        auto h = std::make_unique<pstd_kernel>();
        h->k = std::make_unique<Kernel>();
        if (log_cb) { h->k->logcb = *log_cb; h->k->have_logcb = true; }
        h->k->build(configs, n);
        *out = h.release();
        return PSTD_OK;
    })
}

int pstd_batch_scene(pstd_kernel* h, int32_t scene, int32_t* info) {
    NEED(h);
    auto* k = h->k.get();
    if (scene < 0 || scene >= (int)k->scenes.size()) return fail(PSTD_ERR_INVALID, "scene index out of range");
    info[0] = k->dom_base[scene];
    info[1] = (int32_t)k->scenes[scene].doms.size();
    info[2] = k->rec_base[scene];
    info[3] = (int32_t)k->scenes[scene].receivers.size();
    info[4] = k->scenes[scene].s.framecount();
    return PSTD_OK;
}

int pstd_batch_size(pstd_kernel* h, int32_t* n_scenes, int32_t* n_receivers) {
    NEED(h);
    if (n_scenes) *n_scenes = (int32_t)h->k->scenes.size();
    if (n_receivers) *n_receivers = h->k->n_rec;
    return PSTD_OK;
}

void pstd_destroy(pstd_kernel* k) {
    if (!k) return;
    try { delete k; } catch (...) {}
}

int pstd_get_metadata(pstd_kernel* h, int32_t* n_domains, int32_t* dims, int32_t cap, int32_t* framecount) {
    NEED(h);
    auto* k = h->k.get();
    if (n_domains) *n_domains = (int32_t)k->gdom.size();
    for (int i = 0; i < (int)k->gdom.size() && i < cap && dims; i++) {
        dims[3 * i] = k->dom(i).nx;
        dims[3 * i + 1] = k->dom(i).ny;
        dims[3 * i + 2] = 0;
    }
    if (framecount) *framecount = h->k->framecount;
    return PSTD_OK;
}

int pstd_run(pstd_kernel* h, const pstd_callbacks* cb) {
    NEED_DEVICE(h);
    GUARD({ return run_frames(h->k.get(), cb); })
}

int pstd_run_sub(pstd_kernel* h, const pstd_callbacks* cb, int32_t save_nth, int32_t stride) {
    NEED_DEVICE(h);
    if (save_nth < 0 || stride < 1) return fail(PSTD_ERR_INVALID, "save_nth must be >= 0 and stride >= 1");
    GUARD({ return run_frames(h->k.get(), cb, save_nth, stride); })
}

int pstd_advance(pstd_kernel* h, int32_t n_steps, void* stream) {
    NEED_DEVICE(h);
    if (n_steps < 0) return fail(PSTD_ERR_INVALID, "negative step count");
    GUARD({
        cudaStream_t st = stream ? (cudaStream_t)stream : h->k->stream;
        for (int i = 0; i < n_steps; i++) h->k->step(st);
        return PSTD_OK;
    })
}

int pstd_reset(pstd_kernel* h) {
    NEED_DEVICE(h);
    GUARD({
        CK(cudaDeviceSynchronize());
        h->k->reset();
        return PSTD_OK;
    })
}

int pstd_synchronize(pstd_kernel* h) {
    NEED_DEVICE(h);
    GUARD({
        CK(cudaStreamSynchronize(h->k->stream));
        CK(cudaDeviceSynchronize());
        h->k->check_stage_error();
        return PSTD_OK;
    })
}

int pstd_steps_done(pstd_kernel* h, int32_t* steps) {
    NEED(h);
    *steps = h->k->steps;
    return PSTD_OK;
}

int pstd_get_receivers(pstd_kernel* h, int32_t first_step, int32_t n_steps, float* dst) {
    NEED_DEVICE(h);
    auto* k = h->k.get();
    if (first_step < 0 || n_steps < 0 || first_step + n_steps > k->steps || first_step < k->steps - k->ring_cap)
        return fail(PSTD_ERR_INVALID, "requested receiver steps are not in the device ring");
    if (k->n_rec == 0 || n_steps == 0) return PSTD_OK;
    GUARD({
        CK(cudaDeviceSynchronize());
        for (int s = 0; s < n_steps; s++) {
            int row = (first_step + s) % k->ring_cap;
            CK(cudaMemcpy(dst + (size_t)s * k->n_rec, k->dring.p + (size_t)row * k->n_rec, k->n_rec * sizeof(float),
                          cudaMemcpyDeviceToHost));
        }
        return PSTD_OK;
    })
}

int pstd_snapshot(pstd_kernel* h, int32_t idx, int32_t field, float* dst, int64_t n) {
    NEED_DEVICE(h);
    auto* k = h->k.get();
    if (idx < 0 || idx >= (int)k->hdoms.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const DevDomain& d = k->hdoms[idx];
    const float* base = d.fixed ? k->fixed.p : k->sets[k->cur].p;
    int rows, cols, pitch;
    long long o;
    switch (field) {
        case PSTD_FIELD_P0: rows = d.ny; cols = d.nx; pitch = d.pitch_p; o = d.o_px; break;
        case PSTD_FIELD_PX: rows = d.ny; cols = d.nx; pitch = d.pitch_p; o = d.o_px; break;
        case PSTD_FIELD_PY: rows = d.ny; cols = d.nx; pitch = d.pitch_p; o = d.o_py; break;
        case PSTD_FIELD_VX: rows = d.ny; cols = d.nx + 1; pitch = d.pitch_vx; o = d.o_vx; break;
        case PSTD_FIELD_VY: rows = d.ny + 1; cols = d.nx; pitch = d.pitch_vy; o = d.o_vy; break;
        default: return fail(PSTD_ERR_INVALID, "unknown field code");
    }
    if (n != (int64_t)rows * cols) return fail(PSTD_ERR_INVALID, "destination size does not match the field");
    GUARD({
        CK(cudaDeviceSynchronize());
        if (field == PSTD_FIELD_P0) {
            // the reference's p0 after a step is px + py (kernel/Solver.cpp:114-116),
            // except where it is stale (PML) or initial (no step taken yet)
            if (d.pml || k->steps == 0) {
                CK(cudaMemcpy2D(dst, cols * sizeof(float), k->p0.p + d.o_p0, pitch * sizeof(float), cols * sizeof(float),
                                rows, cudaMemcpyDeviceToHost));
            } else {
                std::vector<float> a((size_t)rows * cols), b((size_t)rows * cols);
                CK(cudaMemcpy2D(a.data(), cols * sizeof(float), base + d.o_px, pitch * sizeof(float), cols * sizeof(float),
                                rows, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy2D(b.data(), cols * sizeof(float), base + d.o_py, pitch * sizeof(float), cols * sizeof(float),
                                rows, cudaMemcpyDeviceToHost));
                for (size_t i = 0; i < a.size(); i++) dst[i] = a[i] + b[i];
            }
        } else {
            CK(cudaMemcpy2D(dst, cols * sizeof(float), base + o, pitch * sizeof(float), cols * sizeof(float), rows,
                            cudaMemcpyDeviceToHost));
        }
        return PSTD_OK;
    })
}

int pstd_scene_strip_runs(pstd_kernel* h, int32_t idx, int32_t axis, int32_t* runs, int32_t cap, int32_t* n) {
    NEED(h);
    auto* k = h->k.get();
    if (idx < 0 || idx >= (int)k->gdom.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const Scene& sc = k->scene_of(idx);
    const int base = k->dom_base[k->gdom[idx].first], local = k->gdom[idx].second;
    int c = 0;
    for (const StripRun& r : sc.runs) {
        if (r.dom != local || (int)r.axis != axis) continue;
        if (c < cap && runs) {
            runs[4 * c] = r.first; runs[4 * c + 1] = r.count;
            runs[4 * c + 2] = r.d1 >= 0 ? base + r.d1 : -1; runs[4 * c + 3] = r.d2 >= 0 ? base + r.d2 : -1;
        }
        c++;
    }
    *n = c;
    return PSTD_OK;
}

int pstd_scene_domain_count(pstd_kernel* h, int32_t* n) {
    NEED(h);
    *n = (int32_t)h->k->gdom.size();
    return PSTD_OK;
}

int pstd_scene_domain_info(pstd_kernel* h, int32_t idx, pstd_domain_info* o) {
    NEED(h);
    auto* k = h->k.get();
    if (idx < 0 || idx >= (int)k->gdom.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const Scene& sc = k->scene_of(idx);
    const Domain& d = k->dom(idx);
    std::memset(o, 0, sizeof *o);
    o->id = d.id;
    o->top_left[0] = d.x0; o->top_left[1] = d.y0;
    o->size[0] = d.nx; o->size[1] = d.ny;
    o->is_pml = d.pml; o->is_secondary_pml = d.secondary; o->is_rigid = d.rigid; o->local = d.local;
    o->should_update[0] = d.update[0]; o->should_update[1] = d.update[1];
    for (int k = 0; k < 4; k++) o->n_neighbours[k] = (int)d.nb[k].size();
    for (int a = 0; a < 2; a++) {
        int n = d.len((Axis)a);
        int W = sc.window_for(n);
        o->window[a] = W;
        o->fft_length[a] = (!d.rigid && d.update[a]) ? Scene::next_pow2(n + 2 * W) : 0;
    }
    o->alpha = d.alpha; o->impedance = d.impedance; o->rho = d.rho;
    return PSTD_OK;
}

int pstd_scene_neighbours(pstd_kernel* h, int32_t idx, int32_t dir, int32_t* out, int32_t cap, int32_t* n) {
    NEED(h);
    auto* k = h->k.get();
    if (idx < 0 || idx >= (int)k->gdom.size() || dir < 0 || dir > 3) return fail(PSTD_ERR_INVALID, "bad index or side");
    const auto& v = k->dom(idx).nb[dir];
    const int base = k->dom_base[k->gdom[idx].first];
    *n = (int32_t)v.size();
    for (int i = 0; i < (int)v.size() && i < cap; i++) out[i] = base + v[i];
    return PSTD_OK;
}

int pstd_scene_attenuation(pstd_kernel* h, int32_t idx, float* ax_p, float* ax_v, float* ay_p, float* ay_v) {
    NEED(h);
    auto* k = h->k.get();
    if (idx < 0 || idx >= (int)k->gdom.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const Scene& sc = k->scene_of(idx);
    const Domain& d = k->dom(idx);
    std::vector<double> prof;
    auto fill = [&](float* dst, int n, bool on, bool vel, bool asc) {
        if (!dst) return;
        if (!on) { for (int i = 0; i < n; i++) dst[i] = 1.f; return; }
        pml_profile(sc.s, vel, asc, prof);
        for (int i = 0; i < n; i++) dst[i] = (float)prof[i];
    };
    fill(ax_p, d.nx, d.pml && d.att_x, false, d.asc_x);
    fill(ax_v, d.nx + 1, d.pml && d.att_x, true, d.asc_x);
    fill(ay_p, d.ny, d.pml && d.att_y, false, d.asc_y);
    fill(ay_v, d.ny + 1, d.pml && d.att_y, true, d.asc_y);
    return PSTD_OK;
}

int pstd_profile_passes(pstd_kernel* h, int32_t n_steps, void* stream, float* ms_stage, float* ms_total,
                        int32_t* stage_launches, int32_t* total_launches) {
    NEED_DEVICE(h);
    GUARD({
        auto* k = h->k.get();
        cudaStream_t st = stream ? (cudaStream_t)stream : k->stream;
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        CK(cudaEventRecord(a, st));
        for (int i = 0; i < n_steps; i++) {
            k->enqueue_step(k->cur, st, true, &ev);   // lengths concurrent, as in the step graphs
            k->cur = (k->cur + 2) % 3;
            k->steps++;
        }
        CK(cudaEventRecord(b, st));
        CK(cudaStreamSynchronize(st));
        float ts = 0, tt = 0;
        for (auto& p : ev) {
            float m;
            CK(cudaEventElapsedTime(&m, p.first, p.second));
            ts += m;
            cudaEventDestroy(p.first);
            cudaEventDestroy(p.second);
        }
        CK(cudaEventElapsedTime(&tt, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (ms_stage) *ms_stage = ts;
        if (ms_total) *ms_total = tt;
        if (stage_launches) *stage_launches = (int32_t)(n_steps * 6 * k->stage_launches().size());
        if (total_launches) *total_launches = n_steps * k->launches_per_step();
        return PSTD_OK;
    })
}

int pstd_work_counts(pstd_kernel* h, int64_t* cells, int64_t* air, int32_t* launches) {
    NEED(h);
    if (cells) *cells = h->k->cells;
    if (air) *air = h->k->air_cells;
    if (launches) *launches = h->k->launches_per_step();
    return PSTD_OK;
}

int pstd_host_register(void* ptr, int64_t bytes) {
    if (!ptr || bytes <= 0) return fail(PSTD_ERR_INVALID, "nothing to register");
    const cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) return fail(PSTD_ERR_CUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
    return PSTD_OK;
}

int pstd_host_unregister(void* ptr) {
    if (!ptr) return fail(PSTD_ERR_INVALID, "nothing to unregister");
    const cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) return fail(PSTD_ERR_CUDA, std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
    return PSTD_OK;
}

int pstd_stage_variants(int32_t L, char* buf, int32_t cap, int32_t* n) {
    const StageVariant* vs;
    const int nv = stage_variants(L, &vs);
    if (n) *n = nv;
    std::string s;
    for (int i = 0; i < nv; i++) s += std::to_string(i) + " " + vs[i].name + "\n";
    if (buf && cap > 0) {
        std::strncpy(buf, s.c_str(), (size_t)cap - 1);
        buf[cap - 1] = 0;
    }
    return PSTD_OK;
}

int pstd_transform_gain(int32_t L, const int32_t* radices, int32_t np, int32_t ctw, int32_t lane_pair, double* out) {
    if (!radices || !out || np < 1 || np > 4 || L < 2) return fail(PSTD_ERR_INVALID, "bad transform description");
    int r[4] = {0, 0, 0, 0}, prod = 1;
    for (int p = 0; p < np; p++) {
        r[p] = radices[p];
        if (r[p] != 2 && r[p] != 4 && r[p] != 8 && r[p] != 16 && r[p] != 32 && !(lane_pair && p == np - 1 && r[p] == 64))
            return fail(PSTD_ERR_INVALID, "radix must be 2, 4, 8, 16 or 32");
        prod *= r[p];
    }
    if (prod != L) return fail(PSTD_ERR_INVALID, "radices do not multiply to L");
    const std::vector<std::complex<double>> g = tgain::round_trip_gain(L, r, np, ctw != 0, lane_pair != 0);
    for (int k = 0; k < L; k++) {
        out[2 * k] = g[k].real();
        out[2 * k + 1] = g[k].imag();
    }
    return PSTD_OK;
}

int pstd_plan_info(pstd_kernel* h, char* buf, int32_t cap) {
    NEED_DEVICE(h);
    std::string s;
    for (auto& b : h->k->buckets) {
        // the variant's index in the length's list (PSTD_PLAN=L:index pins it)
        const StageVariant* vs;
        const int nv = stage_variants(b.L, &vs);
        const long idx = (nv > 0 && b.var >= vs && b.var < vs + nv) ? (long)(b.var - vs) : -1;
        s += "L=" + std::to_string(b.L) + " jobs=" + std::to_string(b.n) + " variant[" + std::to_string(idx) +
             "]=" + b.var->name + b.choice + "\n";
    }
    if (!h->k->form_choice.empty()) s += "form: " + h->k->form_choice + "\n";
    if (h->k->longest_first) s += "order: longest transforms launched first\n";
    if (buf && cap > 0) {
        std::strncpy(buf, s.c_str(), (size_t)cap - 1);
        buf[cap - 1] = 0;
    }
    return PSTD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// pstd_solve_noalloc: the solve of pstd_create + pstd_advance + frame output
// for callers that cannot allocate device memory.  Such callers are host
// applications that own the GPU's memory through their own pool or arena
// (a serving process whose caching allocator has reserved the HBM, an
// acoustics or game engine with a fixed device-memory budget) and real-time
// loops (auralisation) that cannot take cudaMalloc / cudaFree, which may fail
// under the host's budget and synchronise the device.  The caller passes the
// configuration (input) and device buffers for the outputs; everything else
// the solve needs -- the three rotating state sets (the stage kernels'
// scratch), the fixed buffer of rigid domains, p0, the step flag, domain
// table, strip jobs, FP64-derived tables and receiver / speaker lists --
// lives in one file-scope device array of PSTD_NOALLOC_SCRATCH_BYTES.
// ---------------------------------------------------------------------------
namespace pstd {

static __device__ __align__(256) unsigned char g_noalloc_scratch[PSTD_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static constexpr int kNoAllocDevices = 256;
static unsigned char* g_noalloc_base[kNoAllocDevices] = {};

// Device address of the scratch array on the current device.  In host code
// `g_noalloc_scratch` is only a stand-in for the symbol; its address on a
// device comes from cudaGetSymbolAddress, taken once per device (with that
// device current) at the first call on it.
static unsigned char* noalloc_scratch() {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocDevices) throw CudaError("device ordinal out of range for the scratch table");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_base[dev]) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_base[dev] = static_cast<unsigned char*>(p);
    }
    return g_noalloc_base[dev];
}

static int solve_noalloc(const pstd_config* config, int n_steps, float* frame_dev, int64_t frame_len, float* rec_dev,
                         int64_t rec_len, cudaStream_t st) {
    if (!config) return fail(PSTD_ERR_INVALID, "config is NULL");
    if (n_steps < 1) return fail(PSTD_ERR_INVALID, "n_steps must be at least 1");
    if ((frame_len && !frame_dev) || (rec_len && !rec_dev) || frame_len < 0 || rec_len < 0)
        return fail(PSTD_ERR_INVALID, "output pointer is NULL or its length is negative");

    // host-side scene, tables and strip jobs (no device state: nothing here
    // allocates device memory)
    Kernel kh;
    kh.build_scenes(config, 1);
    const Scene& sc = kh.scenes[0];
    const int nd = (int)kh.gdom.size();
    if (sc.spectral) return fail(PSTD_ERR_UNSUPPORTED, "spectral receivers are not available in pstd_solve_noalloc");

    // field layout of pstd_create (device.cuh), from the same function
    const Kernel::FieldLayout lay = kh.layout_fields();
    const std::vector<DevDomain>& hd = lay.doms;
    const std::vector<float>& att = lay.att;
    const std::vector<int>& pml_idx = lay.pml_idx;
    const long long off = (long long)lay.set_floats, foff = (long long)lay.fixed_floats, poff = (long long)lay.p0_floats;
    std::vector<int> x0, y0, frame_doms;
    std::vector<long long> frame_off;
    long long frame_floats = 0;
    for (int k = 0; k < nd; k++) {
        const Domain& d = kh.dom(k);
        if (!d.pml) {
            frame_doms.push_back(k);
            frame_off.push_back(frame_floats);
            frame_floats += (long long)d.nx * d.ny;
        }
        x0.push_back(d.x0);
        y0.push_back(d.y0);
    }

    const int n_rec = (int)sc.receivers.size();
    if (frame_dev && frame_len < frame_floats)
        return fail(PSTD_ERR_INVALID, "frame output holds " + std::to_string(frame_len) + " floats; the scene's frame has " +
                                          std::to_string(frame_floats));
    if (rec_dev && rec_len < (int64_t)n_steps * n_rec)
        return fail(PSTD_ERR_INVALID, "receiver output holds " + std::to_string(rec_len) + " floats; " +
                                          std::to_string(n_steps) + " steps x " + std::to_string(n_rec) +
                                          " receivers are needed");

    // strip-length buckets, each with the first plain variant compiled for it
    struct NB { int L; const StageVariant* var; int off, n, tw; };
    std::vector<NB> nbs;
    for (const StripRun& r : sc.runs) {
        const int L = Kernel::run_length(sc, r);
        bool seen = false;
        for (auto& b : nbs) seen |= b.L == L;
        if (!seen) nbs.push_back({L, nullptr, 0, 0, 0});
    }
    std::sort(nbs.begin(), nbs.end(), [](const NB& a, const NB& b) { return a.L < b.L; });
    std::vector<DevJob> jobs;
    for (size_t i = 0; i < nbs.size(); i++) {
        NB& b = nbs[i];
        const StageVariant* vs;
        const int nv = stage_variants(b.L, &vs);
        // one CTA per job, no staging row cap, FP32 arithmetic
        for (int q = 0; q < nv && !b.var; q++)
            if (!vs[q].persistent && !vs[q].pipe && !vs[q].bf16 && !vs[q].tma) b.var = &vs[q];
        if (!b.var)
            return fail(PSTD_ERR_UNSUPPORTED, "strip transform length " + std::to_string(b.L) +
                                                  " is outside the compiled range 32..8192");
        auto js = kh.make_jobs(b.L, b.var, i + 1 == nbs.size());
        b.off = (int)jobs.size();
        b.n = (int)js.size();
        b.tw = kh.twiddles_of(b.var);
        jobs.insert(jobs.end(), js.begin(), js.end());
    }

    int pml_blocks = 1;   // one block per (row, 128-column chunk) of the largest PML domain
    for (int k : pml_idx) pml_blocks = std::max(pml_blocks, (hd[k].ny + 1) * ((hd[k].nx + 1 + 127) >> 7));

    std::vector<DevReceiver> rec;
    for (auto& r : sc.receivers) rec.push_back({r.dom, r.row, r.col});
    std::vector<DevSpeaker> spk;
    for (auto& q : sc.speakers) spk.push_back({q.x, q.y});

    // carve the scratch array: fields first (cleared every call), then the
    // tables, uploaded every call from one host image
    size_t at = 0;
    auto take = [&](size_t bytes) {
        const size_t o = at;
        at = (at + bytes + 255) / 256 * 256;
        return o;
    };
    const size_t set_bytes = (size_t)std::max<long long>(off, 32) * sizeof(float);
    size_t o_set[3];
    for (auto& o : o_set) o = take(set_bytes);
    const size_t o_fixed = take((size_t)std::max<long long>(foff, 32) * sizeof(float));
    const size_t o_p0 = take((size_t)std::max<long long>(poff, 32) * sizeof(float));
    const size_t o_tab = at;
    const size_t o_flags = take(2 * sizeof(int));   // first-step flag, receiver step counter
    const size_t o_doms = take(hd.size() * sizeof(DevDomain));
    const size_t o_jobs = take(jobs.size() * sizeof(DevJob));
    const size_t o_filt = take(kh.filt.size() * sizeof(float2));
    const size_t o_tw = take(kh.tw.size() * sizeof(float2));
    const size_t o_win = take(kh.win.size() * sizeof(float));
    const size_t o_att = take(att.size() * sizeof(float));
    const size_t o_pml = take(pml_idx.size() * sizeof(int));
    const size_t o_rec = take(rec.size() * sizeof(DevReceiver));
    const size_t o_fdom = take(frame_doms.size() * sizeof(int));
    const size_t o_foff = take(frame_off.size() * sizeof(long long));
    const size_t o_x0 = take(x0.size() * sizeof(int));
    const size_t o_y0 = take(y0.size() * sizeof(int));
    const size_t o_spk = take(spk.size() * sizeof(DevSpeaker));
    if (at > (size_t)PSTD_NOALLOC_SCRATCH_BYTES)
        return fail(PSTD_ERR_INVALID, "scene needs " + std::to_string(at) + " bytes of scratch; pstd_solve_noalloc holds " +
                                          std::to_string((size_t)PSTD_NOALLOC_SCRATCH_BYTES) +
                                          " (PSTD_NOALLOC_SCRATCH_BYTES): use pstd_create for larger scenes");

    std::vector<unsigned char> image(at - o_tab, 0);
    auto put = [&](size_t o, const void* src, size_t bytes) {
        if (bytes) std::memcpy(image.data() + (o - o_tab), src, bytes);
    };
    const int flags[2] = {1, 0};
    put(o_flags, flags, sizeof flags);
    put(o_doms, hd.data(), hd.size() * sizeof(DevDomain));
    put(o_jobs, jobs.data(), jobs.size() * sizeof(DevJob));
    put(o_filt, kh.filt.data(), kh.filt.size() * sizeof(float2));
    put(o_tw, kh.tw.data(), kh.tw.size() * sizeof(float2));
    put(o_win, kh.win.data(), kh.win.size() * sizeof(float));
    put(o_att, att.data(), att.size() * sizeof(float));
    put(o_pml, pml_idx.data(), pml_idx.size() * sizeof(int));
    put(o_rec, rec.data(), rec.size() * sizeof(DevReceiver));
    put(o_fdom, frame_doms.data(), frame_doms.size() * sizeof(int));
    put(o_foff, frame_off.data(), frame_off.size() * sizeof(long long));
    put(o_x0, x0.data(), x0.size() * sizeof(int));
    put(o_y0, y0.data(), y0.size() * sizeof(int));
    put(o_spk, spk.data(), spk.size() * sizeof(DevSpeaker));

    for (const NB& b : nbs) CK(b.var->prepare());
    unsigned char* base = noalloc_scratch();
    auto F = [&](size_t o) { return reinterpret_cast<float*>(base + o); };
    int* first_step = reinterpret_cast<int*>(base + o_flags);
    int* counter = first_step + 1;
    const DevDomain* doms = reinterpret_cast<const DevDomain*>(base + o_doms);
    const DevJob* djobs = reinterpret_cast<const DevJob*>(base + o_jobs);
    const float2* tw = reinterpret_cast<const float2*>(base + o_tw);

    // the array keeps the previous call's contents: clear the fields, then
    // upload this call's tables and flags (first step 1, counter 0); a
    // pageable-source copy returns once the image has been staged
    CK(cudaMemsetAsync(base, 0, o_tab, st));
    CK(cudaMemcpyAsync(base + o_tab, image.data(), image.size(), cudaMemcpyHostToDevice, st));
    if (!spk.empty())
        CK(launch_speakers(doms, reinterpret_cast<const int*>(base + o_x0), reinterpret_cast<const int*>(base + o_y0),
                           nd, reinterpret_cast<const DevSpeaker*>(base + o_spk), (int)spk.size(), sc.s.dx,
                           sc.s.band_width, F(o_set[0]), F(o_fixed), F(o_p0), st));

    int c = 0;
    for (int s = 0; s < n_steps; s++) {
        const int A = (c + 1) % 3, B = (c + 2) % 3;
        for (int k = 0; k < 6; k++) {
            StageArgs a;
            a.doms = doms;
            a.in = F(o_set[k == 0 ? c : ((k - 1) % 2 == 0 ? A : B)]);
            a.prev = F(o_set[c]);
            a.out = F(o_set[k % 2 == 0 ? A : B]);
            a.fixed = F(o_fixed);
            a.p0 = F(o_p0);
            a.first_step = first_step;
            a.filt = a.filt_p = a.filt_v = reinterpret_cast<const float2*>(base + o_filt);
            a.win = F(o_win);
            a.att = F(o_att);
            a.stage = k;
            a.last = k == 5;
            a.row_cap = 0;
            a.maps = nullptr;
            a.set_in = a.set_prev = 0;
            a.err = nullptr;
            for (const NB& b : nbs) {
                a.jobs = djobs + b.off;
                a.tw = tw + b.tw;
                CK(b.var->launch(b.n, a, st));
            }
        }
        if (!pml_idx.empty())
            CK(launch_pml_post(reinterpret_cast<const int*>(base + o_pml), (int)pml_idx.size(), pml_blocks, doms,
                               F(o_set[B]), F(o_fixed), F(o_p0), F(o_att), st));
        CK(cudaMemsetAsync(first_step, 0, sizeof(int), st));
        if (rec_dev && n_rec > 0)
            CK(launch_receivers(reinterpret_cast<const DevReceiver*>(base + o_rec), n_rec, doms, F(o_set[B]), rec_dev,
                                n_steps, counter, st));
        c = B;
    }
    if (frame_dev && !frame_doms.empty())
        CK(launch_frame(reinterpret_cast<const int*>(base + o_fdom), reinterpret_cast<const long long*>(base + o_foff),
                        (int)frame_doms.size(), doms, F(o_set[c]), frame_dev, st));
    return PSTD_OK;
}

}  // namespace pstd

extern "C" int pstd_spectral_plan(const pstd_config* config, int32_t* rows, float* row_weights, float* weights,
                                  int32_t* first, int64_t* sizes) {
    if (!config || !sizes) return fail(PSTD_ERR_INVALID, "config or sizes is NULL");
    GUARD({
        Kernel kh;
        kh.build_scenes(config, 1);
        if (!kh.scenes[0].spectral) throw SceneError(PSTD_ERR_INVALID, "the scene's receivers are not spectral");
        const SpectralPlan plan = kh.spectral_plan();
        const int64_t need[3] = {(int64_t)plan.rows.size(), (int64_t)plan.weights.size(),
                                 (int64_t)plan.first.size() - 1};
        if (rows || row_weights || weights || first) {
            if (sizes[0] < need[0] || sizes[1] < need[1] || sizes[2] < need[2])
                throw SceneError(PSTD_ERR_INVALID, "output arrays smaller than the plan");
            for (size_t i = 0; i < plan.rows.size(); i++) {
                const DevSiRow& q = plan.rows[i];
                const int32_t v[8] = {q.dom, q.row, q.d1, q.d2, q.r1, q.r2, q.W, q.w};
                if (rows) std::memcpy(rows + 8 * i, v, sizeof v);
                if (row_weights) row_weights[i] = q.yw;
            }
            if (weights) std::memcpy(weights, plan.weights.data(), plan.weights.size() * sizeof(float));
            if (first) std::memcpy(first, plan.first.data(), plan.first.size() * sizeof(int32_t));
        }
        for (int j = 0; j < 3; j++) sizes[j] = need[j];
        return 0;
    });
}

extern "C" int pstd_solve_noalloc(const pstd_config* config, int32_t n_steps, float* frame_dev, int64_t frame_len,
                                  float* receivers_dev, int64_t receivers_len, void* stream) {
    GUARD({ return solve_noalloc(config, n_steps, frame_dev, frame_len, receivers_dev, receivers_len,
                                 (cudaStream_t)stream); })
}
