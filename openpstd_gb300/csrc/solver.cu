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
        alloc(std::max<size_t>(v.size(), 1));
        if (!v.empty()) CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
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

// Position of spectrum bin k after the in-place decimation-in-frequency
// transform with radices r[0..np): k = k1 + r1 k2 + r1 r2 k3 + ... sits at
// k1 (L/r1) + k2 (L/(r1 r2)) + ...
static std::vector<int> bin_positions(int L, const int* r, int np) {
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

struct Bucket {
    int L = 0;
    const StageVariant* var = nullptr;
    int off = 0, n = 0;            // jobs in djobs
    int tw_off = 0;                // float2 offset of the twiddles in dtw
    int fp_off = 0, fv_off = 0;    // float2 offsets of the pressure / velocity filters
    int rc = 4;                    // floats staged per strip by the pipelined form
    std::string choice;            // autotune record
};

struct Kernel {
    std::vector<Scene> scenes;          // one per batch member (a single scene: one)
    std::vector<int> dom_base;          // global index of each scene's first domain
    std::vector<int> rec_base;          // global index of each scene's first receiver
    std::vector<std::pair<int, int>> gdom;   // global domain -> (scene, local index)
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> side;     // one per bucket, for concurrent capture
    pstd_callbacks logcb{};
    bool have_logcb = false;
    bool host_only = false;             // built by pstd_scene_build: no device state
    bool autotune = true;
    int smem_optin = 0;                 // largest dynamic shared memory a CTA may opt in to

    // layout
    std::vector<DevDomain> hdoms;
    size_t set_floats = 0, fixed_floats = 0, p0_floats = 0;
    DevBuf<float> sets[3], init_set, fixed, init_fixed, p0, init_p0;
    DevBuf<int> first_step;
    int cur = 0;              // set holding the current (stage-start) state
    int steps = 0;            // steps taken since reset
    int framecount = 0;

    DevBuf<DevDomain> ddoms;
    DevBuf<DevJob> djobs;
    DevBuf<float2> dfilt, dtw;
    DevBuf<float> dwin, datt;
    DevBuf<int> dpml;                 // indices of PML domains
    int n_pml = 0;
    DevBuf<DevReceiver> drec;
    DevBuf<float> dring;
    DevBuf<int> dcounter;
    std::vector<Bucket> buckets;
    int ring_cap = 1;
    int n_rec = 0;
    int64_t cells = 0, air_cells = 0;

    // host-side tables
    std::vector<float> win;
    std::map<std::pair<int, int>, int> win_off;   // (W, patch error)
    std::vector<float2> filt;
    std::map<std::tuple<int, int, int, int, int, int, float>, int> filt_off;   // (L, vel, radices, dx)
    std::vector<float2> tw;
    std::map<std::tuple<int, int, int, int, int>, int> tw_off;   // (L, radices)

    // frames
    std::vector<int> frame_doms;
    std::vector<long long> frame_off;
    size_t frame_floats = 0;
    DevBuf<int> dframe_doms;
    DevBuf<long long> dframe_off;
    DevBuf<float> dframe;

    cudaGraphExec_t graphs[3] = {nullptr, nullptr, nullptr};
    bool graphs_ok = false;

    void log(int level, const std::string& m) {
        if (have_logcb && logcb.log) logcb.log(logcb.user, level, m.c_str());
    }

    ~Kernel() {
        for (auto& g : graphs) if (g) cudaGraphExecDestroy(g);
        for (auto s : side) cudaStreamDestroy(s);
        if (stream) cudaStreamDestroy(stream);
    }

    // ---------------------------------------------------------------- tables
    const Domain& dom(int g) const { return scenes[gdom[g].first].doms[gdom[g].second]; }
    const Scene& scene_of(int g) const { return scenes[gdom[g].first]; }

    int window_of(int W, int patch) {
        auto key = std::make_pair(W, patch);
        auto it = win_off.find(key);
        if (it != win_off.end()) return it->second;
        int o = (int)win.size();
        // kernel/core/kernel_functions.cpp:327-333 (patch error cast to int)
        double walpha = (patch - 40) / 20.0 + 1;
        for (int i = -W; i <= W; i++) {
            double x = (double)i / W;
            double x6 = x * x * x * x * x * x;
            win.push_back((float)std::exp(-std::log(10.0) * walpha * x6));
        }
        win_off[key] = o;
        return o;
    }

    int filter_of(int L, bool vel, const StageVariant* v, float dxf) {
        auto key = std::make_tuple(L, (int)vel, v->r[0], v->r[1], v->r[2], v->r[3], dxf);
        auto it = filt_off.find(key);
        if (it != filt_off.end()) return it->second;
        int o = (int)filt.size();
        // kernel/core/WisdomCache.cpp:53-75: k_j = j (pi/dx)/(L/2) for bins
        // 0..L/2, factor exp(-/+ i k dx/2) * i k; Hermitian extension; 1/L
        const double dx = (double)dxf;
        const double kmax = M_PI / dx;
        std::vector<std::complex<double>> full(L);
        for (int j = 0; j <= L / 2; j++) {
            double k = kmax * j / (L / 2);
            full[j] = std::exp(std::complex<double>(0, (vel ? 0.5 : -0.5) * k * dx)) * std::complex<double>(0, k);
        }
        full[0] = std::complex<double>(full[0].real(), 0);
        full[L / 2] = std::complex<double>(full[L / 2].real(), 0);   // c2r ignores the Nyquist imaginary part
        for (int j = 1; j < L / 2; j++) full[L - j] = std::conj(full[j]);
        std::vector<int> pos = bin_positions(L, v->r, v->np);
        std::vector<float2> perm(L);
        for (int j = 0; j < L; j++) {
            std::complex<double> c = full[j] / (double)L;
            perm[pos[j]] = make_float2((float)c.real(), (float)c.imag());
        }
        filt.insert(filt.end(), perm.begin(), perm.end());
        filt_off[key] = o;
        return o;
    }

    // per-pass twiddle tables of a radix plan: pass p (block size M, radix R)
    // holds [n1][k] = exp(-2 pi i n1 k / M) for n1 < M/R, k < R; the offset
    // of every pass is a multiple of 2 float2 (16-byte loads)
    int twiddles_of(const StageVariant* v) {
        auto key = std::make_tuple(v->L, v->r[0], v->r[1], v->r[2], v->r[3]);
        auto it = tw_off.find(key);
        if (it != tw_off.end()) return it->second;
        if (tw.size() & 1) tw.push_back(make_float2(0, 0));
        int o = (int)tw.size();
        int M = v->L;
        for (int p = 0; p + 1 < v->np; p++) {
            const int R = v->r[p], Q = M / R;
            for (int n1 = 0; n1 < Q; n1++)
                for (int k = 0; k < R; k++) {
                    double a = -2.0 * M_PI * (double)n1 * k / M;
                    tw.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
                }
            M = Q;
        }
        tw_off[key] = o;
        return o;
    }

    static int run_length(const Scene& sc, const StripRun& r) {
        int n = sc.doms[r.dom].len(r.axis);
        return Scene::next_pow2(n + 2 * sc.window_for(n));
    }

    // all jobs of bucket L for variant v (+ copy jobs if `with_copies`);
    // domain indices are global (scene base + local)
    std::vector<DevJob> make_jobs(int L, const StageVariant* v, bool with_copies) {
        std::vector<DevJob> jobs;
        const int per = 2 * v->CS;
        for (size_t si = 0; si < scenes.size(); si++) {
            const Scene& sc = scenes[si];
            const int base = dom_base[si];
            for (const StripRun& r : sc.runs) {
                if (run_length(sc, r) != L) continue;
                const Domain& d = sc.doms[r.dom];
                int n = d.len(r.axis);
                int W = sc.window_for(n);
                int wo = window_of(W, (int)sc.s.patcherror);
                for (int vel = 0; vel < 2; vel++) {
                    // reflection / transmission of the bands (kernel/core/kernel_functions.cpp:37-64)
                    float rs = d.rho;
                    float r1 = r.d1 >= 0 ? sc.doms[r.d1].rho : rs;
                    float r2 = r.d2 >= 0 ? sc.doms[r.d2].rho : rs;
                    float zn1 = r1 / rs, izn1 = rs / r1, zn2 = r2 / rs, izn2 = rs / r2;
                    float rlw1 = (zn1 - 1) / (zn1 + 1), tlw1 = (2 * zn1) / (zn1 + 1), tlw2 = (2 * izn1) / (izn1 + 1);
                    float rrw1 = (zn2 - 1) / (zn2 + 1), trw1 = (2 * zn2) / (zn2 + 1), trw2 = (2 * izn2) / (izn2 + 1);
                    DevJob j;
                    std::memset(&j, 0, sizeof j);
                    j.dom = base + r.dom;
                    j.kind = (vel ? JK_VEL : 0) | (r.axis == AX_Y ? JK_Y : 0);
                    j.W = W;
                    j.d1 = r.d1 >= 0 ? base + r.d1 : -1;
                    j.d2 = r.d2 >= 0 ? base + r.d2 : -1;
                    if (vel) { j.R1 = -rlw1; j.T1 = tlw1; j.R2 = -rrw1; j.T2 = trw1; }
                    else     { j.R1 = rlw1;  j.T1 = tlw2; j.R2 = rrw1;  j.T2 = trw2; }
                    j.dtab = filter_of(L, vel, v, sc.s.dx);
                    j.wtab = wo;
                    int s_ = r.first, end = r.first + r.count;
                    int origin = d.lo(r.axis);
                    while (s_ < end) {
                        int e = std::min(end, (s_ / per + 1) * per);   // cut at multiples of `per`
                        j.first = s_;
                        j.count = e - s_;
                        j.o1 = r.d1 >= 0 ? origin + s_ - sc.doms[r.d1].lo(r.axis) : 0;
                        j.o2 = r.d2 >= 0 ? origin + s_ - sc.doms[r.d2].lo(r.axis) : 0;
                        jobs.push_back(j);
                        s_ = e;
                    }
                }
            }
        }
        if (with_copies) {
            for (size_t g = 0; g < gdom.size(); g++) {
                const Domain& d = dom((int)g);
                if (d.rigid) continue;
                for (int ax = 0; ax < 2; ax++) {
                    if (d.update[ax]) continue;
                    DevJob j;
                    std::memset(&j, 0, sizeof j);
                    j.dom = (int)g;
                    j.kind = JK_COPY | (ax == AX_Y ? JK_Y : 0);
                    j.d1 = j.d2 = -1;
                    jobs.push_back(j);
                }
            }
        }
        return jobs;
    }

    // ---------------------------------------------------------------- build
    void build(const pstd_config* cfgs, int n_cfg) {
        build_scenes(cfgs, n_cfg);
        build_device();
    }

    void build_scenes(const pstd_config* cfgs, int n_cfg) {
        if (n_cfg <= 0) throw SceneError(PSTD_ERR_INVALID, "no scenes");
        scenes.resize(n_cfg);
        for (int i = 0; i < n_cfg; i++) {
            try {
                scenes[i].build(&cfgs[i]);
            } catch (SceneError& e) {
                if (n_cfg == 1) throw;
                throw SceneError(e.code, "scene " + std::to_string(i) + ": " + e.what());
            }
            dom_base.push_back((int)gdom.size());
            for (size_t k = 0; k < scenes[i].doms.size(); k++) gdom.push_back({i, (int)k});
        }
        int nr = 0;
        for (auto& sc : scenes) { rec_base.push_back(nr); nr += (int)sc.receivers.size(); }
        framecount = 0;
        for (auto& sc : scenes) framecount = std::max(framecount, sc.s.framecount());
    }

    void build_device() {
        if (const char* e = std::getenv("PSTD_AUTOTUNE")) autotune = std::atoi(e) != 0;
        // PSTD_VARIANT=i pins every bucket to its i-th compiled variant (tests)
        int forced = -1;
        if (const char* e = std::getenv("PSTD_VARIANT")) { forced = std::atoi(e); autotune = false; }
        CK(cudaGetDevice(&device));
        CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));

        // ---- layout
        auto round32 = [](long long v) { return (v + 31) / 32 * 32; };
        long long off = 0, foff = 0, poff = 0;
        hdoms.resize(gdom.size());
        std::vector<float> att;
        std::vector<int> pml_idx;
        for (size_t k = 0; k < gdom.size(); k++) {
            const Domain& d = dom((int)k);
            const Scene& sc = scene_of((int)k);
            DevDomain& h = hdoms[k];
            std::memset(&h, 0, sizeof h);
            h.nx = d.nx; h.ny = d.ny;
            h.pitch_p = (int)round32(d.nx);
            h.pitch_vx = (int)round32(d.nx + 1);
            h.pitch_vy = (int)round32(d.nx);
            h.fixed = d.rigid;
            h.scene = gdom[k].first;
            long long& o = d.rigid ? foff : off;
            h.o_px = o; o = round32(o + (long long)h.pitch_p * d.ny);
            h.o_py = o; o = round32(o + (long long)h.pitch_p * d.ny);
            h.o_vx = o; o = round32(o + (long long)h.pitch_vx * d.ny);
            h.o_vy = o; o = round32(o + (long long)h.pitch_vy * (d.ny + 1));
            h.o_p0 = poff; poff = round32(poff + (long long)h.pitch_p * d.ny);
            h.rho = d.rho;
            h.c2 = sc.s.c1 * sc.s.c1;
            float dt = sc.s.dt();
            for (int i = 0; i < 6; i++) h.cdt[i] = dt * sc.s.rk[i];
            h.pml = d.pml;
            h.att_xp = h.att_xv = h.att_yp = h.att_yv = -1;
            if (d.pml) {
                pml_idx.push_back((int)k);
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
        fixed_floats = (size_t)std::max<long long>(foff, 32);
        p0_floats = (size_t)std::max<long long>(poff, 32);
        if (att.empty()) att.push_back(1.f);
        datt.upload(att);
        n_pml = (int)pml_idx.size();
        dpml.upload(pml_idx);
        ddoms.upload(hdoms);

        // ---- buckets
        std::vector<int> Ls;
        for (auto& sc : scenes)
            for (const StripRun& r : sc.runs) {
                int L = run_length(sc, r);
                if (std::find(Ls.begin(), Ls.end(), L) == Ls.end()) Ls.push_back(L);
            }
        std::sort(Ls.begin(), Ls.end());
        for (int L : Ls) {
            const StageVariant* vs;
            int nv = stage_variants(L, &vs);
            if (nv <= 0)
                throw SceneError(PSTD_ERR_UNSUPPORTED, "strip transform length " + std::to_string(L) +
                                                           " is outside the compiled range 32..8192");
            for (int i = 0; i < nv; i++) CK(vs[i].prepare());
            Bucket b;
            b.L = L;
            int longest = 0;
            for (auto& sc : scenes)
                for (const StripRun& r : sc.runs)
                    if (run_length(sc, r) == L) longest = std::max(longest, sc.doms[r.dom].len(r.axis));
            b.rc = (longest + 2 + 3) / 4 * 4;
            b.var = &vs[forced >= 0 ? std::min(forced, nv - 1) : 0];
            if (b.var->smem_for(b.rc) > (size_t)smem_optin) b.var = &vs[0];   // pinned form does not fit
            if (forced >= 0) b.choice = " pinned";
            buckets.push_back(b);
        }

        // ---- fields: initial condition
        for (auto& s : sets) s.alloc(set_floats);
        init_set.alloc(set_floats);
        fixed.alloc(fixed_floats);
        init_fixed.alloc(fixed_floats);
        p0.alloc(p0_floats);
        init_p0.alloc(p0_floats);
        first_step.alloc(scenes.size());
        CK(cudaMemsetAsync(init_set.p, 0, set_floats * sizeof(float), stream));
        CK(cudaMemsetAsync(init_fixed.p, 0, fixed_floats * sizeof(float), stream));
        CK(cudaMemsetAsync(init_p0.p, 0, p0_floats * sizeof(float), stream));
        {
            std::vector<int> x0, y0;
            for (size_t g = 0; g < gdom.size(); g++) { x0.push_back(dom((int)g).x0); y0.push_back(dom((int)g).y0); }
            DevBuf<int> dx0, dy0;
            dx0.upload(x0);
            dy0.upload(y0);
            for (size_t si = 0; si < scenes.size(); si++) {
                const Scene& sc = scenes[si];
                if (sc.speakers.empty()) continue;
                std::vector<DevSpeaker> spk;
                for (auto& q : sc.speakers) spk.push_back({q.x, q.y});
                DevBuf<DevSpeaker> dspk;
                dspk.upload(spk);
                const int b = dom_base[si];
                CK(launch_speakers(ddoms.p + b, dx0.p + b, dy0.p + b, (int)sc.doms.size(), dspk.p, (int)spk.size(),
                                   sc.s.dx, sc.s.band_width, init_set.p, init_fixed.p, init_p0.p, stream));
                CK(cudaStreamSynchronize(stream));
            }
        }

        // ---- receivers, frames
        std::vector<DevReceiver> rec;
        for (size_t si = 0; si < scenes.size(); si++)
            for (auto& r : scenes[si].receivers) rec.push_back({dom_base[si] + r.dom, r.row, r.col});
        n_rec = (int)rec.size();
        drec.upload(rec);
        ring_cap = std::max(framecount, 1);
        dring.alloc((size_t)ring_cap * std::max(n_rec, 1));
        dcounter.alloc(1);
        frame_floats = 0;
        for (size_t k = 0; k < gdom.size(); k++) {
            if (dom((int)k).pml) continue;
            frame_doms.push_back((int)k);
            frame_off.push_back((long long)frame_floats);
            frame_floats += (size_t)dom((int)k).nx * dom((int)k).ny;
        }
        dframe_doms.upload(frame_doms);
        dframe_off.upload(frame_off);
        dframe.alloc(std::max<size_t>(frame_floats, 1));

        // ---- tables and the job plan (autotuned)
        reset();
        plan(autotune);
        reset();
        for (size_t i = 0; i < buckets.size(); i++) {
            cudaStream_t s;
            CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            side.push_back(s);
        }
        capture_graphs();
        std::string choice;
        for (auto& b : buckets) choice += " [" + std::string(b.var->name) + b.choice + "]";
        log(PSTD_LOG_DEBUG, std::to_string(scenes.size()) + " scene(s), " + std::to_string(gdom.size()) + " domains, " +
                                std::to_string(n_rec) + " receivers; stage kernels:" + choice);
    }

    StageArgs stage_args(int c, int k, const DevJob* jobs, const float2* twp, int fp, int fv, int rc) {
        const int A = (c + 1) % 3, B = (c + 2) % 3;
        StageArgs a;
        a.jobs = jobs;
        a.doms = ddoms.p;
        a.in = sets[k == 0 ? c : ((k - 1) % 2 == 0 ? A : B)].p;
        a.prev = sets[c].p;
        a.out = sets[k % 2 == 0 ? A : B].p;
        a.fixed = fixed.p;
        a.p0 = p0.p;
        a.first_step = first_step.p;
        a.filt = dfilt.p;
        a.filt_p = dfilt.p + fp;
        a.filt_v = dfilt.p + fv;
        a.win = dwin.p;
        a.tw = twp;
        a.att = datt.p;
        a.stage = k;
        a.last = k == 5;
        a.row_cap = rc;
        return a;
    }

    void upload_tables() {
        dfilt.upload(filt);
        dtw.upload(tw);
        dwin.upload(win);
    }

    // the persistent form stages one pressure / velocity filter pair per CTA
    static bool one_filter_pair(const std::vector<DevJob>& jobs, int fp, int fv) {
        for (const DevJob& j : jobs)
            if (!(j.kind & JK_COPY) && j.dtab != ((j.kind & JK_VEL) ? fv : fp)) return false;
        return true;
    }

    // choose a variant per bucket by timing each on this batch's jobs
    void plan(bool tune) {
        if (tune) {
            for (auto& b : buckets) {
                const StageVariant* vs;
                int nv = stage_variants(b.L, &vs);
                if (nv <= 1) continue;
                std::vector<std::vector<DevJob>> all(nv);
                std::vector<int> twv(nv), fpv(nv), fvv(nv);
                for (int i = 0; i < nv; i++) {
                    all[i] = make_jobs(b.L, &vs[i], false);
                    twv[i] = twiddles_of(&vs[i]);
                    fpv[i] = filter_of(b.L, false, &vs[i], scenes[0].s.dx);
                    fvv[i] = filter_of(b.L, true, &vs[i], scenes[0].s.dx);
                    if (vs[i].persistent && !one_filter_pair(all[i], fpv[i], fvv[i])) all[i].clear();
                    if (vs[i].smem_for(b.rc) > (size_t)smem_optin) all[i].clear();   // staging too large
                }
                upload_tables();
                float best = 1e30f;
                int best_i = 0;
                std::string rec;
                cudaEvent_t e0, e1;
                CK(cudaEventCreate(&e0));
                CK(cudaEventCreate(&e1));
                for (int i = 0; i < nv; i++) {
                    if (all[i].empty()) continue;
                    DevBuf<DevJob> tj;
                    tj.upload(all[i]);
                    StageArgs a = stage_args(cur, 1, tj.p, dtw.p + twv[i], fpv[i], fvv[i], b.rc);
                    if (vs[i].launch((int)all[i].size(), a, stream) != cudaSuccess) {
                        cudaGetLastError();   // this variant's staging does not fit the bucket's strips
                        rec += " " + std::to_string(i) + ":n/a";
                        continue;
                    }
                    CK(vs[i].launch((int)all[i].size(), a, stream));
                    CK(cudaEventRecord(e0, stream));
                    const int reps = 5;
                    for (int w = 0; w < reps; w++) CK(vs[i].launch((int)all[i].size(), a, stream));
                    CK(cudaEventRecord(e1, stream));
                    CK(cudaEventSynchronize(e1));
                    float ms;
                    CK(cudaEventElapsedTime(&ms, e0, e1));
                    ms /= reps;
                    char buf[64];
                    std::snprintf(buf, sizeof buf, " %d:%.1fus", i, ms * 1e3f);
                    rec += buf;
                    if (ms < best) { best = ms; best_i = i; }
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                b.var = &vs[best_i];
                b.choice = " tuned" + rec;
            }
        }
        std::vector<DevJob> jobs;
        for (size_t i = 0; i < buckets.size(); i++) {
            auto& b = buckets[i];
            auto js = make_jobs(b.L, b.var, i + 1 == buckets.size());
            b.tw_off = twiddles_of(b.var);
            b.fp_off = filter_of(b.L, false, b.var, scenes[0].s.dx);
            b.fv_off = filter_of(b.L, true, b.var, scenes[0].s.dx);
            if (b.var->persistent && !one_filter_pair(js, b.fp_off, b.fv_off)) {
                // mixed grid spacings: fall back to the first plain variant
                const StageVariant* vs;
                int nv = stage_variants(b.L, &vs);
                for (int q = 0; q < nv; q++) if (!vs[q].persistent) { b.var = &vs[q]; break; }
                js = make_jobs(b.L, b.var, i + 1 == buckets.size());
                b.tw_off = twiddles_of(b.var);
                b.choice += " (plain: several grid spacings)";
            }
            b.off = (int)jobs.size();
            b.n = (int)js.size();
            jobs.insert(jobs.end(), js.begin(), js.end());
        }
        upload_tables();
        djobs.upload(jobs);
    }

    void reset() {
        for (auto& s : sets) CK(cudaMemsetAsync(s.p, 0, set_floats * sizeof(float), stream));
        CK(cudaMemcpyAsync(sets[0].p, init_set.p, set_floats * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(fixed.p, init_fixed.p, fixed_floats * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(p0.p, init_p0.p, p0_floats * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        std::vector<int> ones(scenes.size(), 1);
        CK(cudaMemcpy(first_step.p, ones.data(), ones.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemsetAsync(dcounter.p, 0, sizeof(int), stream));
        CK(cudaStreamSynchronize(stream));
        cur = 0;
        steps = 0;
    }

    int launches_per_step() const { return 6 * (int)buckets.size() + (n_pml > 0) + 1; }

    // Enqueue one time step from set `c` on `st`.  concurrent: the buckets of
    // a stage go on side streams (fork/join); ev (optional): events around
    // each stage's launches, which then run back to back on `st`.
    void enqueue_step(int c, cudaStream_t st, bool concurrent,
                      std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* ev = nullptr) {
        const int B = (c + 2) % 3;
        std::vector<cudaEvent_t> tmp;
        auto mk = [&]() {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            tmp.push_back(e);
            return e;
        };
        for (int k = 0; k < 6; k++) {
            cudaEvent_t t0 = nullptr, t1 = nullptr;
            if (ev) {
                CK(cudaEventCreate(&t0));
                CK(cudaEventCreate(&t1));
                CK(cudaEventRecord(t0, st));
            }
            if (concurrent && buckets.size() > 1) {
                cudaEvent_t fork = mk();
                CK(cudaEventRecord(fork, st));
                std::vector<cudaEvent_t> joins;
                for (size_t i = 0; i < buckets.size(); i++) {
                    auto& b = buckets[i];
                    cudaStream_t s = i == 0 ? st : side[i];
                    if (i > 0) CK(cudaStreamWaitEvent(s, fork, 0));
                    StageArgs a = stage_args(c, k, djobs.p + b.off, dtw.p + b.tw_off, b.fp_off, b.fv_off, b.rc);
                    CK(b.var->launch(b.n, a, s));
                    if (i > 0) {
                        cudaEvent_t j = mk();
                        CK(cudaEventRecord(j, s));
                        joins.push_back(j);
                    }
                }
                for (auto j : joins) CK(cudaStreamWaitEvent(st, j, 0));
            } else {
                for (auto& b : buckets) {
                    StageArgs a = stage_args(c, k, djobs.p + b.off, dtw.p + b.tw_off, b.fp_off, b.fv_off, b.rc);
                    CK(b.var->launch(b.n, a, st));
                }
            }
            if (ev) {
                CK(cudaEventRecord(t1, st));
                ev->push_back({t0, t1});
            }
        }
        if (n_pml > 0) CK(launch_pml_post(dpml.p, n_pml, ddoms.p, sets[B].p, fixed.p, p0.p, datt.p, st));
        CK(cudaMemsetAsync(first_step.p, 0, scenes.size() * sizeof(int), st));
        CK(launch_receivers(drec.p, n_rec, ddoms.p, sets[B].p, dring.p, ring_cap, dcounter.p, st));
        for (auto e : tmp) cudaEventDestroy(e);   // destruction is deferred until the event completes
    }

    void capture_graphs() {
        graphs_ok = false;
        bool ok = true;
        for (int c = 0; c < 3 && ok; c++) {
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { ok = false; break; }
            try {
                enqueue_step(c, stream, true);
            } catch (...) {
                cudaStreamEndCapture(stream, &g);
                if (g) cudaGraphDestroy(g);
                ok = false;
                break;
            }
            if (cudaStreamEndCapture(stream, &g) != cudaSuccess || !g) { ok = false; break; }
            if (cudaGraphInstantiate(&graphs[c], g, 0) != cudaSuccess) { cudaGraphDestroy(g); ok = false; break; }
            cudaGraphDestroy(g);
        }
        cudaGetLastError();
        graphs_ok = ok;
        if (!ok) log(PSTD_LOG_WARNING, "CUDA graph capture failed; launching kernels directly");
    }

    void step(cudaStream_t st) {
        if (graphs_ok) CK(cudaGraphLaunch(graphs[cur], st));
        else enqueue_step(cur, st, false);
        cur = (cur + 2) % 3;
        steps++;
    }
};

static int run_frames(Kernel* k, const pstd_callbacks* cb) {
    if (k->scenes.size() != 1) throw SceneError(PSTD_ERR_INVALID, "run() delivers frames of a single scene; advance batches");
    const Scene& sc = k->scenes[0];
    const int nframes = k->framecount;
    const int save = std::max(1, sc.s.save_nth);
    const size_t frame_floats = k->frame_floats;
    const int K = 3;   // frames in flight
    const size_t slot = frame_floats + (size_t)std::max(k->n_rec, 1);
    PinnedBuf stage;
    stage.alloc(slot * K);
    std::vector<cudaEvent_t> ev(K);
    for (auto& e : ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    struct Pending { int frame, slot; };
    std::deque<Pending> q;
    int status = PSTD_OK;
    auto log = [&](int lvl, const std::string& m) { if (cb && cb->log) cb->log(cb->user, lvl, m.c_str()); };
    auto deliver = [&](const Pending& p) {
        CK(cudaEventSynchronize(ev[p.slot]));
        float* base = stage.p + slot * p.slot;
        for (size_t i = 0; i < k->frame_doms.size(); i++) {
            int d = k->frame_doms[i];
            size_t n = (size_t)k->hdoms[d].nx * k->hdoms[d].ny;
            if (cb && cb->write_frame && status == PSTD_OK)
                if (cb->write_frame(cb->user, p.frame, sc.doms[d].id, base + k->frame_off[i], (int64_t)n) != 0)
                    status = PSTD_ERR_CALLBACK;
        }
        for (int r = 0; r < k->n_rec; r++) {
            if (cb && cb->write_sample && status == PSTD_OK)
                if (cb->write_sample(cb->user, p.frame, sc.receivers[r].id, base + frame_floats + r, 1) != 0)
                    status = PSTD_ERR_CALLBACK;
        }
        log(PSTD_LOG_INFO, "Finished frame: " + std::to_string(p.frame));
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
            if (frame_floats) {
                CK(launch_frame(k->dframe_doms.p, k->dframe_off.p, (int)k->frame_doms.size(), k->ddoms.p,
                                k->sets[k->cur].p, k->dframe.p, k->stream));
                CK(cudaMemcpyAsync(base, k->dframe.p, frame_floats * sizeof(float), cudaMemcpyDeviceToHost, k->stream));
            }
            if (k->n_rec > 0) {
                int row = (k->steps - 1) % k->ring_cap;
                CK(cudaMemcpyAsync(base + frame_floats, k->dring.p + (size_t)row * k->n_rec, k->n_rec * sizeof(float),
                                   cudaMemcpyDeviceToHost, k->stream));
            }
            CK(cudaEventRecord(ev[s], k->stream));
            q.push_back({f, s});
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
            k->enqueue_step(k->cur, st, false, &ev);
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
        if (stage_launches) *stage_launches = (int32_t)(n_steps * 6 * k->buckets.size());
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

int pstd_plan_info(pstd_kernel* h, char* buf, int32_t cap) {
    NEED_DEVICE(h);
    std::string s;
    for (auto& b : h->k->buckets)
        s += "L=" + std::to_string(b.L) + " jobs=" + std::to_string(b.n) + " variant=" + b.var->name + b.choice + "\n";
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

    // field layout of pstd_create (device.cuh)
    auto round32 = [](long long v) { return (v + 31) / 32 * 32; };
    long long off = 0, foff = 0, poff = 0;
    std::vector<DevDomain> hd(nd);
    std::vector<float> att;
    std::vector<int> pml_idx, x0, y0, frame_doms;
    std::vector<long long> frame_off;
    long long frame_floats = 0;
    for (int k = 0; k < nd; k++) {
        const Domain& d = kh.dom(k);
        DevDomain& h = hd[k];
        std::memset(&h, 0, sizeof h);
        h.nx = d.nx; h.ny = d.ny;
        h.pitch_p = (int)round32(d.nx);
        h.pitch_vx = (int)round32(d.nx + 1);
        h.pitch_vy = (int)round32(d.nx);
        h.fixed = d.rigid;
        h.scene = 0;
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
            pml_idx.push_back(k);
            std::vector<double> prof;
            auto put = [&](bool vel, bool asc, int& at) {
                pml_profile(sc.s, vel, asc, prof);
                at = (int)att.size();
                for (double v : prof) att.push_back((float)v);
            };
            if (d.att_x) { put(false, d.asc_x, h.att_xp); put(true, d.asc_x, h.att_xv); }
            if (d.att_y) { put(false, d.asc_y, h.att_yp); put(true, d.asc_y, h.att_yv); }
        } else {
            frame_doms.push_back(k);
            frame_off.push_back(frame_floats);
            frame_floats += (long long)d.nx * d.ny;
        }
        x0.push_back(d.x0);
        y0.push_back(d.y0);
    }
    if (att.empty()) att.push_back(1.f);

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
        for (int q = 0; q < nv && !b.var; q++) if (!vs[q].persistent) b.var = &vs[q];
        if (!b.var)
            return fail(PSTD_ERR_UNSUPPORTED, "strip transform length " + std::to_string(b.L) +
                                                  " is outside the compiled range 32..8192");
        auto js = kh.make_jobs(b.L, b.var, i + 1 == nbs.size());
        b.off = (int)jobs.size();
        b.n = (int)js.size();
        b.tw = kh.twiddles_of(b.var);
        jobs.insert(jobs.end(), js.begin(), js.end());
    }

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
            for (const NB& b : nbs) {
                a.jobs = djobs + b.off;
                a.tw = tw + b.tw;
                CK(b.var->launch(b.n, a, st));
            }
        }
        if (!pml_idx.empty())
            CK(launch_pml_post(reinterpret_cast<const int*>(base + o_pml), (int)pml_idx.size(), doms, F(o_set[B]),
                               F(o_fixed), F(o_p0), F(o_att), st));
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

extern "C" int pstd_solve_noalloc(const pstd_config* config, int32_t n_steps, float* frame_dev, int64_t frame_len,
                                  float* receivers_dev, int64_t receivers_len, void* stream) {
    GUARD({ return solve_noalloc(config, n_steps, frame_dev, frame_len, receivers_dev, receivers_len,
                                 (cudaStream_t)stream); })
}
