// solver.cu -- host runtime of the GB300 PSTD solve and the C ABI of
// include/pstd_gb300.h.
//
// pstd_create builds the scene on the host (scene.cpp), the FP64 tables
// (window, derivative filters, twiddles, PML profiles), the device field
// layout (device.cuh) and the strip-job plan, then uploads everything once.
// A time step is 12 strip passes (x then y for each of the 6 RK stages,
// kernel/Solver.cpp:77-79,95-117) plus one receiver gather; the three phases
// of the state-set rotation are captured as three CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pstd_gb300.h"
#include "launch.hpp"
#include "scene.hpp"

namespace pstd {

static thread_local std::string g_error;

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

#define CK(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        release();
        n = count;
        if (count) CK(cudaMalloc(&p, count * sizeof(T)));
    }
    void upload(const std::vector<T>& v) {
        alloc(v.size());
        if (!v.empty()) CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
};

struct Group {     // one pass launch: jobs of one strip length
    int L;
    int offset, count;
};

// position of spectrum bin k after the in-place decimation-in-frequency
// transform with radices r[0..np): k = k1 + r1 k2 + r1 r2 k3 + ... sits at
// k1 (L/r1) + k2 (L/(r1 r2)) + ...
static std::vector<int> bin_positions(int L) {
    int r[4], np;
    pass_radices(L, r, &np);
    std::vector<int> pos(L);
    for (int k = 0; k < L; k++) {
        int rem = k, span = L, p = 0;
        for (int i = 0; i < np; i++) {
            int d = rem % r[i];
            rem /= r[i];
            span /= r[i];
            p += d * span;
        }
        pos[k] = p;
    }
    return pos;
}

struct Kernel {
    Scene sc;
    int device = 0;
    cudaStream_t stream = nullptr;
    pstd_callbacks logcb{};
    bool have_logcb = false;

    // layout
    std::vector<DevDomain> hdoms;
    size_t set_floats = 0;
    DevBuf<float> sets[3];
    DevBuf<float> init_set;
    int cur = 0;              // set holding the current (stage-start) state
    int steps = 0;            // steps taken since reset
    int framecount = 0;

    DevBuf<DevDomain> ddoms;
    DevBuf<DevJob> djobs;
    DevBuf<DevCopy> dcopies;
    DevBuf<float2> dfilt, dtw;
    DevBuf<float> dwin, datt;
    DevBuf<DevReceiver> drec;
    DevBuf<float> dring;
    DevBuf<int> dcounter;
    std::map<int, int> tw_offset;   // L -> float2 offset in dtw
    std::vector<Group> xgroups, ygroups;
    int xcopy_off = 0, xcopy_n = 0, ycopy_off = 0, ycopy_n = 0;
    int ring_cap = 1;
    int n_rec = 0;
    int64_t cells = 0, air_cells = 0;

    cudaGraphExec_t graphs[3] = {nullptr, nullptr, nullptr};
    bool graphs_ok = false;

    void log(int level, const std::string& m) {
        if (have_logcb && logcb.log) logcb.log(logcb.user, level, m.c_str());
    }

    ~Kernel() {
        for (auto& g : graphs) if (g) cudaGraphExecDestroy(g);
        if (stream) cudaStreamDestroy(stream);
    }

    void build(const pstd_config* cfg) {
        sc.build(cfg);
        framecount = sc.s.framecount();
        CK(cudaGetDevice(&device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CK(prepare_pass_kernels());

        // ---- layout
        auto round32 = [](long long v) { return (v + 31) / 32 * 32; };
        long long off = 0;
        hdoms.resize(sc.doms.size());
        std::vector<float> att;
        for (size_t k = 0; k < sc.doms.size(); k++) {
            const Domain& d = sc.doms[k];
            DevDomain& h = hdoms[k];
            std::memset(&h, 0, sizeof h);
            h.nx = d.nx; h.ny = d.ny;
            h.pitch_p = (int)round32(d.nx);
            h.pitch_vx = (int)round32(d.nx + 1);
            h.pitch_vy = (int)round32(d.nx);
            h.o_p0 = off; off = round32(off + (long long)h.pitch_p * d.ny);
            h.o_px = off; off = round32(off + (long long)h.pitch_p * d.ny);
            h.o_py = off; off = round32(off + (long long)h.pitch_p * d.ny);
            h.o_vx = off; off = round32(off + (long long)h.pitch_vx * d.ny);
            h.o_vy = off; off = round32(off + (long long)h.pitch_vy * (d.ny + 1));
            h.rho = d.rho;
            h.c2 = sc.s.c1 * sc.s.c1;
            float dt = sc.s.dt();
            for (int i = 0; i < 6; i++) h.cdt[i] = dt * sc.s.rk[i];
            h.pml = d.pml;
            h.att_xp = h.att_xv = h.att_yp = h.att_yv = -1;
            if (d.pml) {
                std::vector<double> prof;
                if (d.att_x) {
                    pml_profile(sc.s, false, d.asc_x, prof);
                    h.att_xp = (int)att.size(); for (double v : prof) att.push_back((float)v);
                    pml_profile(sc.s, true, d.asc_x, prof);
                    h.att_xv = (int)att.size(); for (double v : prof) att.push_back((float)v);
                }
                if (d.att_y) {
                    pml_profile(sc.s, false, d.asc_y, prof);
                    h.att_yp = (int)att.size(); for (double v : prof) att.push_back((float)v);
                    pml_profile(sc.s, true, d.asc_y, prof);
                    h.att_yv = (int)att.size(); for (double v : prof) att.push_back((float)v);
                }
            }
            if (!d.rigid) cells += (int64_t)d.nx * d.ny;
            if (!d.pml) air_cells += (int64_t)d.nx * d.ny;
        }
        set_floats = (size_t)std::max<long long>(off, 32);
        if (att.empty()) att.push_back(1.f);
        datt.upload(att);

        // ---- tables: windows, derivative filters, twiddles
        std::map<int, int> win_off;            // W -> offset
        std::vector<float> win;
        std::map<std::pair<int, int>, int> filt_off;   // (L, velocity) -> offset
        std::vector<float2> filt, tw;
        auto window_of = [&](int W) {
            auto it = win_off.find(W);
            if (it != win_off.end()) return it->second;
            int o = (int)win.size();
            // kernel/core/kernel_functions.cpp:327-333, patch error cast to int
            double walpha = ((int)sc.s.patcherror - 40) / 20.0 + 1;
            for (int i = -W; i <= W; i++) {
                double x = (double)i / W;
                double x6 = x * x * x * x * x * x;
                win.push_back((float)std::exp(-std::log(10.0) * walpha * x6));
            }
            win_off[W] = o;
            return o;
        };
        auto filter_of = [&](int L, bool vel) {
            auto key = std::make_pair(L, (int)vel);
            auto it = filt_off.find(key);
            if (it != filt_off.end()) return it->second;
            int o = (int)filt.size();
            // kernel/core/WisdomCache.cpp:53-75: k_j = j (pi/dx)/(L/2), factor
            // exp(-/+ i k dx/2) * i k for bins 0..L/2, Hermitian extension, /L
            const double dx = (double)sc.s.dx;
            const double kmax = M_PI / dx;
            std::vector<std::complex<double>> full(L);
            for (int j = 0; j <= L / 2; j++) {
                double k = kmax * j / (L / 2);
                std::complex<double> ik(0, k);
                std::complex<double> shift = std::exp(std::complex<double>(0, (vel ? 0.5 : -0.5) * k * dx));
                full[j] = shift * ik;
            }
            full[0] = std::complex<double>(full[0].real(), 0);
            full[L / 2] = std::complex<double>(full[L / 2].real(), 0);   // c2r ignores the Nyquist imaginary part
            for (int j = 1; j < L / 2; j++) full[L - j] = std::conj(full[j]);
            std::vector<int> pos = bin_positions(L);
            std::vector<float2> perm(L);
            for (int j = 0; j < L; j++) {
                std::complex<double> v = full[j] / (double)L;
                perm[pos[j]] = make_float2((float)v.real(), (float)v.imag());
            }
            filt.insert(filt.end(), perm.begin(), perm.end());
            filt_off[key] = o;
            return o;
        };
        auto twiddles_of = [&](int L) {
            if (tw_offset.count(L)) return;
            tw_offset[L] = (int)tw.size();
            for (int j = 0; j < L; j++) {
                double a = -2.0 * M_PI * j / L;
                tw.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
            }
        };

        // ---- jobs
        std::map<int, std::vector<DevJob>> xj, yj;
        for (const StripRun& r : sc.runs) {
            const Domain& d = sc.doms[r.dom];
            int n = d.len(r.axis);
            int W = sc.window_for(n);
            int L = Scene::next_pow2(n + 2 * W);
            int per = pass_strips_per_job(L);
            if (per <= 0)
                throw SceneError(PSTD_ERR_UNSUPPORTED, "strip transform length " + std::to_string(L) + " is not supported (32..8192)");
            twiddles_of(L);
            int wo = window_of(W);
            for (int vel = 0; vel < 2; vel++) {
                int fo = filter_of(L, vel);
                // reflection/transmission of the two bands (kernel/core/kernel_functions.cpp:37-64)
                float rs = d.rho;
                float r1 = r.d1 >= 0 ? sc.doms[r.d1].rho : rs;
                float r2 = r.d2 >= 0 ? sc.doms[r.d2].rho : rs;
                float zn1 = r1 / rs, izn1 = rs / r1, zn2 = r2 / rs, izn2 = rs / r2;
                float rlw1 = (zn1 - 1) / (zn1 + 1), tlw1 = (2 * zn1) / (zn1 + 1), tlw2 = (2 * izn1) / (izn1 + 1);
                float rrw1 = (zn2 - 1) / (zn2 + 1), trw1 = (2 * zn2) / (zn2 + 1), trw2 = (2 * izn2) / (izn2 + 1);
                DevJob j;
                std::memset(&j, 0, sizeof j);
                j.dom = r.dom;
                j.kind = (vel ? JK_VEL : 0) | (r.axis == AX_Y ? JK_Y : 0);
                j.W = W;
                j.d1 = r.d1; j.d2 = r.d2;
                if (vel) { j.R1 = -rlw1; j.T1 = tlw1; j.R2 = -rrw1; j.T2 = trw1; }
                else     { j.R1 = rlw1;  j.T1 = tlw2; j.R2 = rrw1;  j.T2 = trw2; }
                j.dtab = fo;
                j.wtab = wo;
                // cut the run at multiples of `per` strips (relative to the domain)
                int s = r.first, end = r.first + r.count;
                while (s < end) {
                    int e = std::min(end, (s / per + 1) * per);
                    j.first = s;
                    j.count = e - s;
                    int origin = d.lo(r.axis);   // global strip coordinate of strip 0
                    j.o1 = r.d1 >= 0 ? origin + s - sc.doms[r.d1].lo(r.axis) : 0;
                    j.o2 = r.d2 >= 0 ? origin + s - sc.doms[r.d2].lo(r.axis) : 0;
                    (r.axis == AX_X ? xj : yj)[L].push_back(j);
                    s = e;
                }
            }
        }
        std::vector<DevJob> jobs;
        for (auto* m : {&xj, &yj}) {
            for (auto& kv : *m) {
                Group g{kv.first, (int)jobs.size(), (int)kv.second.size()};
                jobs.insert(jobs.end(), kv.second.begin(), kv.second.end());
                (m == &xj ? xgroups : ygroups).push_back(g);
            }
        }
        std::vector<DevCopy> copies;
        for (size_t k = 0; k < sc.doms.size(); k++)
            if (sc.doms[k].rigid || !sc.doms[k].update[AX_X]) copies.push_back({(int)k, 0});
        xcopy_off = 0; xcopy_n = (int)copies.size();
        for (size_t k = 0; k < sc.doms.size(); k++)
            if (sc.doms[k].rigid || !sc.doms[k].update[AX_Y]) copies.push_back({(int)k, JK_Y});
        ycopy_off = xcopy_n; ycopy_n = (int)copies.size() - xcopy_n;
        if (jobs.empty()) jobs.push_back(DevJob{});
        if (copies.empty()) copies.push_back(DevCopy{0, 0});
        if (filt.empty()) filt.push_back(make_float2(0, 0));
        if (tw.empty()) tw.push_back(make_float2(1, 0));
        if (win.empty()) win.push_back(1.f);

        ddoms.upload(hdoms);
        djobs.upload(jobs);
        dcopies.upload(copies);
        dfilt.upload(filt);
        dtw.upload(tw);
        dwin.upload(win);

        // ---- receivers
        std::vector<DevReceiver> rec;
        for (auto& r : sc.receivers) rec.push_back({r.dom, r.row, r.col});
        n_rec = (int)rec.size();
        if (rec.empty()) rec.push_back({0, 0, 0});
        drec.upload(rec);
        ring_cap = std::max(framecount, 1);
        dring.alloc((size_t)ring_cap * std::max(n_rec, 1));
        dcounter.alloc(1);

        // ---- fields: initial condition into init_set, then copy
        for (auto& s : sets) s.alloc(set_floats);
        init_set.alloc(set_floats);
        CK(cudaMemsetAsync(init_set.p, 0, set_floats * sizeof(float), stream));
        if (!sc.speakers.empty()) {
            std::vector<int> x0, y0;
            for (auto& d : sc.doms) { x0.push_back(d.x0); y0.push_back(d.y0); }
            DevBuf<int> dx0, dy0;
            dx0.upload(x0);
            dy0.upload(y0);
            std::vector<DevSpeaker> spk;
            for (auto& s : sc.speakers) spk.push_back({s.x, s.y});
            DevBuf<DevSpeaker> dspk;
            dspk.upload(spk);
            CK(launch_speakers(ddoms.p, dx0.p, dy0.p, (int)sc.doms.size(), dspk.p, (int)spk.size(), sc.s.dx,
                               sc.s.band_width, init_set.p, stream));
            CK(cudaStreamSynchronize(stream));
        }
        reset();
        CK(cudaStreamSynchronize(stream));
        capture_graphs();
        log(PSTD_LOG_DEBUG, "scene: " + std::to_string(sc.doms.size()) + " domains, " + std::to_string(sc.speakers.size()) +
                                " speakers, " + std::to_string(sc.receivers.size()) + " receivers");
    }

    void reset() {
        for (auto& s : sets) CK(cudaMemsetAsync(s.p, 0, set_floats * sizeof(float), stream));
        CK(cudaMemcpyAsync(sets[0].p, init_set.p, set_floats * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemsetAsync(dcounter.p, 0, sizeof(int), stream));
        cur = 0;
        steps = 0;
    }

    int launches_per_step() const {
        int per_stage = (int)xgroups.size() + (int)ygroups.size() + (xcopy_n > 0) + (ycopy_n > 0);
        return 6 * per_stage + 1;
    }

    // enqueue one time step starting from set `c`; events (optional) bracket
    // the x and y pass launches for timing
    void enqueue_step(int c, cudaStream_t st, std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* xev = nullptr,
                      std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* yev = nullptr) {
        const int A = (c + 1) % 3, B = (c + 2) % 3;
        for (int k = 0; k < 6; k++) {
            const float* in = sets[k == 0 ? c : ((k - 1) % 2 == 0 ? A : B)].p;
            float* out = sets[k % 2 == 0 ? A : B].p;
            PassArgs a{nullptr, ddoms.p, in, sets[c].p, out, dfilt.p, dwin.p, nullptr, datt.p, k, k == 5};
            for (int dir = 0; dir < 2; dir++) {
                auto& groups = dir == 0 ? xgroups : ygroups;
                auto* ev = dir == 0 ? xev : yev;
                cudaEvent_t e0 = nullptr, e1 = nullptr;
                if (ev) {
                    CK(cudaEventCreate(&e0));
                    CK(cudaEventCreate(&e1));
                    CK(cudaEventRecord(e0, st));
                }
                for (const Group& g : groups) {
                    a.jobs = djobs.p + g.offset;
                    a.tw = dtw.p + tw_offset[g.L];
                    CK(launch_pass(g.L, g.count, a, st));
                }
                if (ev) {
                    CK(cudaEventRecord(e1, st));
                    ev->push_back({e0, e1});
                }
                int co = dir == 0 ? xcopy_off : ycopy_off, cn = dir == 0 ? xcopy_n : ycopy_n;
                CK(launch_copy(dcopies.p + co, cn, ddoms.p, sets[c].p, out, datt.p, k == 5, st));
            }
        }
        CK(launch_receivers(drec.p, n_rec, ddoms.p, sets[B].p, dring.p, ring_cap, dcounter.p, st));
    }

    void capture_graphs() {
        graphs_ok = false;
        cudaStream_t cs;
        CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        bool ok = true;
        for (int c = 0; c < 3 && ok; c++) {
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { ok = false; break; }
            try {
                enqueue_step(c, cs);
            } catch (...) {
                cudaStreamEndCapture(cs, &g);
                if (g) cudaGraphDestroy(g);
                ok = false;
                break;
            }
            if (cudaStreamEndCapture(cs, &g) != cudaSuccess || !g) { ok = false; break; }
            if (cudaGraphInstantiate(&graphs[c], g, 0) != cudaSuccess) { cudaGraphDestroy(g); ok = false; break; }
            cudaGraphDestroy(g);
        }
        cudaStreamDestroy(cs);
        cudaGetLastError();
        graphs_ok = ok;
        if (!ok) log(PSTD_LOG_WARNING, "CUDA graph capture failed; launching kernels directly");
    }

    void step(cudaStream_t st) {
        if (graphs_ok) CK(cudaGraphLaunch(graphs[cur], st));
        else enqueue_step(cur, st);
        cur = (cur + 2) % 3;
        steps++;
    }

    // p0 of a domain from the current set into a dense host buffer
    void copy_p0(int k, float* dst, cudaStream_t st) {
        const DevDomain& h = hdoms[k];
        CK(cudaMemcpy2DAsync(dst, h.nx * sizeof(float), sets[cur].p + h.o_p0, h.pitch_p * sizeof(float),
                             h.nx * sizeof(float), h.ny, cudaMemcpyDeviceToHost, st));
    }
};

struct PinnedBuf {
    float* p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        if (count <= n) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        CK(cudaMallocHost(&p, count * sizeof(float)));
        n = count;
    }
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
};

static int run_frames(Kernel* k, const pstd_callbacks* cb) {
    const int nframes = k->framecount;
    const int save = std::max(1, k->sc.s.save_nth);
    std::vector<int> emit_doms;
    size_t frame_floats = 0;
    for (size_t d = 0; d < k->sc.doms.size(); d++)
        if (!k->sc.doms[d].pml) { emit_doms.push_back((int)d); frame_floats += (size_t)k->hdoms[d].nx * k->hdoms[d].ny; }
    const int K = 3;   // frames in flight
    const size_t slot = frame_floats + (size_t)std::max(k->n_rec, 1);
    PinnedBuf stage;
    stage.alloc(slot * K);
    std::vector<cudaEvent_t> ev(K);
    for (auto& e : ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    struct Pending { int frame, slot, step; };
    std::deque<Pending> q;
    int status = PSTD_OK;
    auto log = [&](int lvl, const std::string& m) { if (cb && cb->log) cb->log(cb->user, lvl, m.c_str()); };
    auto deliver = [&](const Pending& p) {
        CK(cudaEventSynchronize(ev[p.slot]));
        float* base = stage.p + slot * p.slot;
        size_t o = 0;
        for (int d : emit_doms) {
            size_t n = (size_t)k->hdoms[d].nx * k->hdoms[d].ny;
            if (cb && cb->write_frame && status == PSTD_OK)
                if (cb->write_frame(cb->user, p.frame, k->sc.doms[d].id, base + o, (int64_t)n) != 0) status = PSTD_ERR_CALLBACK;
            o += n;
        }
        for (int r = 0; r < k->n_rec; r++) {
            if (cb && cb->write_sample && status == PSTD_OK)
                if (cb->write_sample(cb->user, p.frame, k->sc.receivers[r].id, base + frame_floats + r, 1) != 0)
                    status = PSTD_ERR_CALLBACK;
        }
        log(PSTD_LOG_INFO, "Finished frame: " + std::to_string(p.frame));
    };
    log(PSTD_LOG_DEBUG, "Number of render time: " + std::to_string(k->sc.s.calctime));
    log(PSTD_LOG_DEBUG, "Size of time step: " + std::to_string(k->sc.s.dt()));
    log(PSTD_LOG_INFO, "Starting simulation");
    int next_slot = 0;
    for (int f = 0; f < nframes && status == PSTD_OK; f++) {
        k->step(k->stream);
        if (f % save == 0) {
            int s = next_slot;
            next_slot = (next_slot + 1) % K;
            float* base = stage.p + slot * s;
            size_t o = 0;
            for (int d : emit_doms) {
                k->copy_p0(d, base + o, k->stream);
                o += (size_t)k->hdoms[d].nx * k->hdoms[d].ny;
            }
            if (k->n_rec > 0) {
                int row = (k->steps - 1) % k->ring_cap;
                CK(cudaMemcpyAsync(base + frame_floats, k->dring.p + (size_t)row * k->n_rec, k->n_rec * sizeof(float),
                                   cudaMemcpyDeviceToHost, k->stream));
            }
            CK(cudaEventRecord(ev[s], k->stream));
            q.push_back({f, s, k->steps});
        } else {
            log(PSTD_LOG_INFO, "Finished frame: " + std::to_string(f));
        }
        while ((int)q.size() >= K) { deliver(q.front()); q.pop_front(); }
    }
    while (!q.empty()) {
        if (status == PSTD_OK) deliver(q.front());
        q.pop_front();
    }
    CK(cudaStreamSynchronize(k->stream));
    for (auto& e : ev) cudaEventDestroy(e);
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

extern "C" {

const char* pstd_last_error(void) { return g_error.c_str(); }
const char* pstd_version(void) { return "pstd_gb300 0.1.0 (sm_103a)"; }

int pstd_create(const pstd_config* config, const pstd_callbacks* log_cb, pstd_kernel** out) {
    if (!out) return fail(PSTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    GUARD({
        auto h = std::make_unique<pstd_kernel>();
        h->k = std::make_unique<Kernel>();
        if (log_cb) { h->k->logcb = *log_cb; h->k->have_logcb = true; }
        h->k->log(PSTD_LOG_DEBUG, "Initializing kernel");
        h->k->build(config);
        h->k->log(PSTD_LOG_DEBUG, "Finished initializing kernel");
        *out = h.release();
        return PSTD_OK;
    })
}

void pstd_destroy(pstd_kernel* k) {
    if (!k) return;
    try { delete k; } catch (...) {}
}

int pstd_get_metadata(pstd_kernel* h, int32_t* n_domains, int32_t* dims, int32_t cap, int32_t* framecount) {
    NEED(h);
    auto& sc = h->k->sc;
    if (n_domains) *n_domains = (int32_t)sc.doms.size();
    for (int i = 0; i < (int)sc.doms.size() && i < cap && dims; i++) {
        dims[3 * i] = sc.doms[i].nx;
        dims[3 * i + 1] = sc.doms[i].ny;
        dims[3 * i + 2] = 0;
    }
    if (framecount) *framecount = h->k->framecount;
    return PSTD_OK;
}

int pstd_run(pstd_kernel* h, const pstd_callbacks* cb) {
    NEED(h);
    GUARD({ return run_frames(h->k.get(), cb); })
}

int pstd_advance(pstd_kernel* h, int32_t n_steps, void* stream) {
    NEED(h);
    if (n_steps < 0) return fail(PSTD_ERR_INVALID, "negative step count");
    GUARD({
        cudaStream_t st = stream ? (cudaStream_t)stream : h->k->stream;
        for (int i = 0; i < n_steps; i++) h->k->step(st);
        return PSTD_OK;
    })
}

int pstd_reset(pstd_kernel* h) {
    NEED(h);
    GUARD({
        h->k->reset();
        return PSTD_OK;
    })
}

int pstd_synchronize(pstd_kernel* h) {
    NEED(h);
    GUARD({
        CK(cudaStreamSynchronize(h->k->stream));
        CK(cudaDeviceSynchronize());
        return PSTD_OK;
    })
}

int pstd_steps_done(pstd_kernel* h, int32_t* steps) {
    NEED(h);
    *steps = h->k->steps;
    return PSTD_OK;
}

int pstd_get_receivers(pstd_kernel* h, int32_t first_step, int32_t n_steps, float* dst) {
    NEED(h);
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
    NEED(h);
    auto* k = h->k.get();
    if (idx < 0 || idx >= (int)k->hdoms.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const DevDomain& d = k->hdoms[idx];
    int rows, cols, pitch;
    long long o;
    switch (field) {
        case PSTD_FIELD_P0: rows = d.ny; cols = d.nx; pitch = d.pitch_p; o = d.o_p0; break;
        case PSTD_FIELD_PX: rows = d.ny; cols = d.nx; pitch = d.pitch_p; o = d.o_px; break;
        case PSTD_FIELD_PY: rows = d.ny; cols = d.nx; pitch = d.pitch_p; o = d.o_py; break;
        case PSTD_FIELD_VX: rows = d.ny; cols = d.nx + 1; pitch = d.pitch_vx; o = d.o_vx; break;
        case PSTD_FIELD_VY: rows = d.ny + 1; cols = d.nx; pitch = d.pitch_vy; o = d.o_vy; break;
        default: return fail(PSTD_ERR_INVALID, "unknown field code");
    }
    if (n != (int64_t)rows * cols) return fail(PSTD_ERR_INVALID, "destination size does not match the field");
    GUARD({
        CK(cudaDeviceSynchronize());
        CK(cudaMemcpy2D(dst, cols * sizeof(float), k->sets[k->cur].p + o, pitch * sizeof(float), cols * sizeof(float),
                        rows, cudaMemcpyDeviceToHost));
        return PSTD_OK;
    })
}

int pstd_scene_domain_count(pstd_kernel* h, int32_t* n) {
    NEED(h);
    *n = (int32_t)h->k->sc.doms.size();
    return PSTD_OK;
}

int pstd_scene_domain_info(pstd_kernel* h, int32_t idx, pstd_domain_info* o) {
    NEED(h);
    auto& sc = h->k->sc;
    if (idx < 0 || idx >= (int)sc.doms.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const Domain& d = sc.doms[idx];
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
    auto& sc = h->k->sc;
    if (idx < 0 || idx >= (int)sc.doms.size() || dir < 0 || dir > 3) return fail(PSTD_ERR_INVALID, "bad index or side");
    const auto& v = sc.doms[idx].nb[dir];
    *n = (int32_t)v.size();
    for (int i = 0; i < (int)v.size() && i < cap; i++) out[i] = v[i];
    return PSTD_OK;
}

int pstd_scene_attenuation(pstd_kernel* h, int32_t idx, float* ax_p, float* ax_v, float* ay_p, float* ay_v) {
    NEED(h);
    auto& sc = h->k->sc;
    if (idx < 0 || idx >= (int)sc.doms.size()) return fail(PSTD_ERR_INVALID, "domain index out of range");
    const Domain& d = sc.doms[idx];
    std::vector<double> prof;
    auto fill = [&](float* dst, int n, bool on, bool vel, bool asc) {
        if (!dst) return;
        if (!on) { for (int i = 0; i < n; i++) dst[i] = 1.f; return; }
        pml_profile(sc.s, vel, asc, prof);
        for (int i = 0; i < n; i++) dst[i] = (float)prof[i];
    };
    bool pml = d.pml;
    fill(ax_p, d.nx, pml && d.att_x, false, d.asc_x);
    fill(ax_v, d.nx + 1, pml && d.att_x, true, d.asc_x);
    fill(ay_p, d.ny, pml && d.att_y, false, d.asc_y);
    fill(ay_v, d.ny + 1, pml && d.att_y, true, d.asc_y);
    return PSTD_OK;
}

int pstd_profile_passes(pstd_kernel* h, int32_t n_steps, void* stream, float* ms_x, float* ms_y, int32_t* lx,
                        int32_t* ly) {
    NEED(h);
    GUARD({
        auto* k = h->k.get();
        cudaStream_t st = stream ? (cudaStream_t)stream : k->stream;
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> xe, ye;
        for (int i = 0; i < n_steps; i++) {
            k->enqueue_step(k->cur, st, &xe, &ye);
            k->cur = (k->cur + 2) % 3;
            k->steps++;
        }
        CK(cudaStreamSynchronize(st));
        float tx = 0, ty = 0;
        for (auto& p : xe) { float m; CK(cudaEventElapsedTime(&m, p.first, p.second)); tx += m; cudaEventDestroy(p.first); cudaEventDestroy(p.second); }
        for (auto& p : ye) { float m; CK(cudaEventElapsedTime(&m, p.first, p.second)); ty += m; cudaEventDestroy(p.first); cudaEventDestroy(p.second); }
        if (ms_x) *ms_x = tx;
        if (ms_y) *ms_y = ty;
        if (lx) *lx = (int32_t)(n_steps * 6 * k->xgroups.size());
        if (ly) *ly = (int32_t)(n_steps * 6 * k->ygroups.size());
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

}  // extern "C"
