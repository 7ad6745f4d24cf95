// kernel_state.hpp -- the solver's host-side state (scene batch, FP64-built
// tables, device field layout, strip-job plan, CUDA graphs) shared by the C
// ABI of solver.cu and the serving loop of server.cu.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "transform_gain.hpp"
#include "../../include/pstd_gb300.h"
#include "launch.hpp"
#include "scene.hpp"
#include "spectral_receivers.hpp"

namespace pstd {

// record the message of a failing C-ABI call (pstd_last_error) and return code
int set_error(int code, const std::string& message);

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

// PSTD_DFT selects a tensor-core DFT precision study for the strip lengths
// that have one: "bf16x3" (split BF16 on mma.sync) or "tf32x3" (split TF32 on
// tcgen05 with TMEM accumulators); the default is the FP32 FFT
inline std::string study_dft() {
    const char* e = std::getenv("PSTD_DFT");
    return e ? std::string(e) : std::string();
}
inline bool want_bf16_dft() {
    const std::string s = study_dft();
    return s == "bf16x3" || s == "tf32x3";
}
inline bool study_variant_matches(const StageVariant& v) {
    const std::string s = study_dft();
    return v.bf16 && ((s == "tf32x3") == v.tc5);
}

// the FP32 variants come first in every list; the study variants follow
inline int fp32_variants(const StageVariant* vs, int nv) {
    int n = 0;
    while (n < nv && !vs[n].bf16) n++;
    return n;
}

// PSTD_GAIN_COMPENSATION=0 builds the derivative filters without dividing by
// the transform's round-trip gain (for measuring what the division buys)
inline bool gain_compensation() {
    static const bool on = [] {
        const char* e = std::getenv("PSTD_GAIN_COMPENSATION");
        return !e || std::atoi(e) != 0;
    }();
    return on;
}

// PSTD_PLAN="L:i,L:i,..." pins the variant of each listed strip length (for
// profiling a plan the autotuner chose without a profiler); -1 = not listed.
// PSTD_PLAN=serving pins every length to the plain variant with the
// configuration of the serving loop's per-length persistent form.
inline int planned_variant(int L) {
    const char* e = std::getenv("PSTD_PLAN");
    if (!e) return -1;
    std::string s(e);
    if (s == "serving") {
        const StageVariant* sv = serve_variant(L);
        const StageVariant* vs;
        const int nv = stage_variants(L, &vs);
        for (int i = 0; sv && i < nv; i++) {
            const StageVariant& v = vs[i];
            if (v.CS == sv->CS && v.NT == sv->NT && v.smem == sv->smem && v.ctw == sv->ctw && v.shf == 0 &&
                !v.persistent && !v.pipe && !v.bf16 && !v.tma && !v.tc5 && v.r[0] == sv->r[0] && v.r[1] == sv->r[1] &&
                v.r[2] == sv->r[2] && v.r[3] == sv->r[3])
                return i;
        }
        return -1;
    }
    size_t at = 0;
    while (at < s.size()) {
        size_t end = s.find(',', at);
        if (end == std::string::npos) end = s.size();
        const std::string item = s.substr(at, end - at);
        const size_t c = item.find(':');
        if (c != std::string::npos && std::atoi(item.substr(0, c).c_str()) == L) return std::atoi(item.c_str() + c + 1);
        at = end + 1;
    }
    return -1;
}

// Plans chosen by the autotuner, kept per process and keyed by the scene's
// strip-job structure (like the reference's WisdomCache for FFT plans): a scene
// tuned once is created again without timing.
struct PlanChoice {
    std::vector<std::pair<int, const StageVariant*>> vars;   // (L, variant)
    bool merged = false;
    int merged_fam = 0;
    bool longest_first = false;
    std::string form;
};
inline std::mutex& plan_cache_mutex() {
    static std::mutex m;
    return m;
}
inline std::map<std::string, PlanChoice>& plan_cache() {
    static std::map<std::string, PlanChoice> c;
    return c;
}

struct Bucket {
    int L = 0;
    const StageVariant* var = nullptr;
    int off = 0, n = 0;            // jobs in djobs
    int tw_off = 0;                // float2 offset of the twiddles in dtw
    int fp_off = 0, fv_off = 0;    // float2 offsets of the pressure / velocity filters
    int rc = 4;                    // floats staged per strip by the pipelined form
    bool pinned = false;           // variant fixed by PSTD_PLAN / PSTD_DFT: not tuned
    std::vector<const StageVariant*> cands;   // fastest variants timed alone (refined on whole steps)
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
    int pml_blocks = 0;               // grid of the PML post kernel
    DevBuf<int> dpml_off;             // prefix sums of its blocks per PML domain

    // one block per (row, 128-column chunk) of every PML domain, in one flat grid
    void set_pml_blocks(const std::vector<int>& pml) {
        std::vector<int> off{0};
        for (int k : pml) off.push_back(off.back() + (hdoms[k].ny + 1) * ((hdoms[k].nx + 1 + 127) >> 7));
        pml_blocks = off.back();
        dpml_off.upload(off);
    }
    DevBuf<DevReceiver> drec;
    DevBuf<float> dring;
    DevBuf<int> dcounter;
    // spectral receivers: stencil rows, their weights, first row per receiver, row values
    bool spectral = false;
    int n_si_rows = 0;
    DevBuf<DevSiRow> dsi_rows;
    DevBuf<float> dsi_w, dsi_val;
    DevBuf<int> dsi_first;
    std::vector<Bucket> buckets;
    int ring_cap = 1;
    int n_rec = 0;
    int64_t cells = 0, air_cells = 0;

    // host-side tables
    std::vector<float> win;
    std::map<std::pair<int, int>, int> win_off;   // (W, patch error)
    std::vector<float2> filt;
    std::map<std::tuple<int, int, int, int, int, int, float, int>, int> filt_off;   // (L, vel, radices, dx, form)
    std::vector<float2> tw;
    std::map<std::tuple<int, int, int, int, int, int>, int> tw_off;   // (L, radices, lane-pair split / computed twiddles)

    // frames
    std::vector<int> frame_doms;
    std::vector<long long> frame_off;
    size_t frame_floats = 0;
    DevBuf<int> dframe_doms;
    DevBuf<long long> dframe_off;
    // run()'s frame slots (device) and their pinned host staging, kept across
    // runs; made at create for frames of up to 8 slots in 128 MiB
    PinnedBuf run_stage;
    DevBuf<float> run_slots;
    // frames in flight of run() for slots of `slot` floats: up to 8 within 64 MiB, at least 3
    static int run_slot_count(size_t slot) {
        return (int)std::min<size_t>(8, std::max<size_t>(3, (size_t(64) << 20) / (std::max<size_t>(slot, 1) * sizeof(float))));
    }
    void reserve_run_slots(size_t floats) {
        run_stage.alloc(floats);
        if (run_slots.n < floats) run_slots.alloc(floats);
    }

    // staged (TMA) form: a 2-D tensor map per (domain, field, state set) and
    // the error word a CTA sets when a staged copy does not arrive in time
    DevBuf<unsigned char> dmaps;
    DevBuf<int> derr;

    cudaGraphExec_t graphs[3] = {nullptr, nullptr, nullptr};
    bool graphs_ok = false;

    // serving loop (server.cu): first-step flags per slot, receivers into
    // per-scene rings at per-scene step counts
    struct ServerHooks {
        bool on = false;
        int n_flags = 0;
        const DevSrvReceiver* rec = nullptr;
        float* aux = nullptr;
        int* scene_step = nullptr;
        const int* limit = nullptr;   // per slot: the scene's step count
        const int* slots = nullptr;
        int n_slots = 0;
    } srv;

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

    // The derivative filter of a variant: the reference's factors, 1/L, and the
    // division by the round-trip gain of the variant's transform per bin
    // (transform_gain.hpp; the tensor-core study forms are left as they are).
    // Direct-convolution forms (v->direct = Q) take the real kernel h of the
    // same factors instead, extended to 2L + Q floats: hx[e] = h[(e - L) mod L].
    int filter_of(int L, bool vel, const StageVariant* v, float dxf) {
        const bool study = v->bf16 || v->tc5;
        const int form = v->direct ? 8 + v->direct : study ? 3 : (v->shf ? 2 : 0) + (v->ctw ? 1 : 0) * 4;
        auto key = std::make_tuple(L, (int)vel, v->r[0], v->r[1], v->r[2], v->r[3], dxf, form);
        auto it = filt_off.find(key);
        if (it != filt_off.end()) return it->second;
        int o = (int)filt.size();
        std::vector<std::complex<double>> gain(L, std::complex<double>(1, 0));
        if (!study && gain_compensation()) gain = tgain::round_trip_gain(L, v->r, v->np, v->ctw != 0, v->shf != 0);
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
        if (v->direct) {
            // h[d] = (1/L) sum_k D[k] exp(2 pi i k d / L) (real: D is Hermitian)
            std::vector<double> h(L);
            for (int d = 0; d < L; d++) {
                double acc = 0;
                for (int k = 0; k < L; k++) {
                    const double a = 2.0 * M_PI * (double)(((long long)k * d) % L) / L;
                    acc += full[k].real() * std::cos(a) - full[k].imag() * std::sin(a);
                }
                h[d] = acc / L;
            }
            const int ne = 2 * L + v->direct;
            std::vector<float> hx(ne + (ne & 1), 0.f);
            for (int e = 0; e < ne; e++) hx[e] = (float)h[((e - L) % L + L) % L];
            for (size_t e = 0; e < hx.size(); e += 2) filt.push_back(make_float2(hx[e], hx[e + 1]));
            filt_off[key] = o;
            return o;
        }
        std::vector<int> pos = bin_positions(L, v->r, v->np);
        std::vector<float2> perm(L);
        for (int j = 0; j < L; j++) {
            std::complex<double> c = full[j] / (double)L / gain[j];
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
        auto key = std::make_tuple(v->L, v->r[0], v->r[1], v->r[2], v->r[3], v->shf * 2 + v->ctw);
        auto it = tw_off.find(key);
        if (it != tw_off.end()) return it->second;
        if (tw.size() & 1) tw.push_back(make_float2(0, 0));
        int o = (int)tw.size();
        int M = v->L;
        auto put = [&](double n, int M_) {
            double a = -2.0 * M_PI * n / M_;
            tw.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
        };
        for (int p = 0; p + 1 < v->np; p++) {
            const int R = v->r[p], Q = M / R;
            for (int n1 = 0; n1 < Q; n1++) {
                if (!v->ctw) {
                    for (int k = 0; k < R; k++) put((double)n1 * k, M);
                } else if (R >= 16) {   // the powers make_twiddles multiplies out (stage_kernel.cuh)
                    put(n1, M); put(2.0 * n1, M); put(4.0 * n1, M); put(8.0 * n1, M);
                } else if (R == 8) {
                    put(n1, M); put(4.0 * n1, M);
                } else if (R == 4) {
                    put(n1, M); put(2.0 * n1, M);
                } else {
                    put(n1, M); put(n1, M);
                }
            }
            M = Q;
        }
        if (v->shf) {
            // last radix 2H over a lane pair: H ones (lane 0), then exp(-2 pi i j / 2H), j < H (lane 1)
            const int H = M / 2;
            for (int j = 0; j < H; j++) tw.push_back(make_float2(1.f, 0.f));
            for (int j = 0; j < H; j++) {
                double a = -2.0 * M_PI * (double)j / M;
                tw.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
            }
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
                    DevJob j;
                    std::memset(&j, 0, sizeof j);
                    j.dom = base + r.dom;
                    j.kind = (vel ? JK_VEL : 0) | (r.axis == AX_Y ? JK_Y : 0);
                    j.W = W;
                    j.d1 = r.d1 >= 0 ? base + r.d1 : -1;
                    j.d2 = r.d2 >= 0 ? base + r.d2 : -1;
                    band_coefficients(d.rho, r.d1 >= 0 ? sc.doms[r.d1].rho : d.rho, r.d2 >= 0 ? sc.doms[r.d2].rho : d.rho,
                                      vel != 0, j.R1, j.T1, j.R2, j.T2);
                    j.dtab = filter_of(L, vel, v, sc.s.dx);
                    j.wtab = wo;
                    j.L = L;
                    j.ttab = twiddles_of(v);
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

    // stencils of the spectral receivers of every scene (host tables only)
    SpectralPlan spectral_plan() {
        SpectralPlan plan;
        for (size_t si = 0; si < scenes.size(); si++)
            plan_spectral_receivers(scenes[si], dom_base[si], [&](int W) {
                const int o = window_of(W, (int)scenes[si].s.patcherror);   // may grow the table: first
                return win.data() + o;
            }, plan);
        plan.first.push_back((int)plan.rows.size());
        return plan;
    }

    // Layout of every domain's fields in a state set, the fixed buffer and the
    // p0 array (device.cuh: rows padded to 32 floats, each field starting on a
    // 128-byte boundary), the PML attenuation profiles and the PML domains.
    // pstd_create and the allocation-free solve both use it.
    struct FieldLayout {
        std::vector<DevDomain> doms;
        std::vector<float> att;      // never empty
        std::vector<int> pml_idx;
        size_t set_floats = 0, fixed_floats = 0, p0_floats = 0;
    };
    // Offsets, pitches and constants of one domain in the layout of
    // device.cuh.  off / foff / poff: the next free float of the state set,
    // the fixed buffer and the p0 array (advanced past the domain); the
    // attenuation offsets are left at -1 for the caller.
    static void layout_domain(const Domain& d, const Scene& sc, int scene, long long& off, long long& foff,
                              long long& poff, DevDomain& h) {
        auto round32 = [](long long v) { return (v + 31) / 32 * 32; };
        std::memset(&h, 0, sizeof h);
        h.nx = d.nx; h.ny = d.ny;
        h.pitch_p = (int)round32(d.nx);
        h.pitch_vx = (int)round32(d.nx + 1);
        h.pitch_vy = (int)round32(d.nx);
        h.fixed = d.rigid;
        h.scene = scene;
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
    }

    FieldLayout layout_fields() const {
        long long off = 0, foff = 0, poff = 0;
        FieldLayout out;
        out.doms.resize(gdom.size());
        for (size_t k = 0; k < gdom.size(); k++) {
            const Domain& d = dom((int)k);
            const Scene& sc = scene_of((int)k);
            DevDomain& h = out.doms[k];
            layout_domain(d, sc, gdom[k].first, off, foff, poff, h);
            if (d.pml) {
                out.pml_idx.push_back((int)k);
                std::vector<double> prof;
                auto put = [&](bool vel, bool asc, int& at) {
                    pml_profile(sc.s, vel, asc, prof);
                    at = (int)out.att.size();
                    for (double v : prof) out.att.push_back((float)v);
                };
                if (d.att_x) { put(false, d.asc_x, h.att_xp); put(true, d.asc_x, h.att_xv); }
                if (d.att_y) { put(false, d.asc_y, h.att_yp); put(true, d.asc_y, h.att_yv); }
            }
        }
        out.set_floats = (size_t)std::max<long long>(off, 32);
        out.fixed_floats = (size_t)std::max<long long>(foff, 32);
        out.p0_floats = (size_t)std::max<long long>(poff, 32);
        if (out.att.empty()) out.att.push_back(1.f);
        return out;
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
        FieldLayout lay = layout_fields();
        hdoms = lay.doms;
        std::vector<float>& att = lay.att;
        std::vector<int>& pml_idx = lay.pml_idx;
        for (size_t k = 0; k < gdom.size(); k++) {
            const Domain& d = dom((int)k);
            if (!d.rigid) cells += (int64_t)d.nx * d.ny;
            if (!d.pml) air_cells += (int64_t)d.nx * d.ny;
        }
        set_floats = lay.set_floats;
        fixed_floats = lay.fixed_floats;
        p0_floats = lay.p0_floats;
        datt.upload(att);
        n_pml = (int)pml_idx.size();
        dpml.upload(pml_idx);
        set_pml_blocks(pml_idx);
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
            const int nv_fp32 = fp32_variants(vs, nv);
            b.var = &vs[forced >= 0 ? std::min(forced, nv_fp32 - 1) : 0];
            if (b.var->smem_for(b.rc) > (size_t)smem_optin) b.var = &vs[0];   // pinned form does not fit
            if (want_bf16_dft())
                for (int i = 0; i < nv; i++)
                    if (study_variant_matches(vs[i])) {
                        b.var = &vs[i];
                        b.choice = vs[i].tc5 ? " split-TF32 tcgen05 DFT (precision study)"
                                             : " split-BF16 DFT (precision study)";
                        b.pinned = true;
                    }
            if (int i = planned_variant(L); i >= 0 && i < nv_fp32) {
                b.var = &vs[i];
                b.choice = " pinned by PSTD_PLAN";
                b.pinned = true;
            }
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
        derr.alloc(1);
        CK(cudaMemset(derr.p, 0, sizeof(int)));
        build_tensor_maps();
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
        spectral = scenes[0].spectral;
        for (auto& sc : scenes)
            if (sc.spectral != spectral)
                throw SceneError(PSTD_ERR_UNSUPPORTED, "a batch mixes spectral and nearest-neighbour receivers");
        if (spectral) {
            const SpectralPlan plan = spectral_plan();
            n_si_rows = (int)plan.rows.size();
            dsi_rows.upload(plan.rows);
            dsi_w.upload(plan.weights);
            dsi_first.upload(plan.first);
            dsi_val.alloc((size_t)std::max(n_si_rows, 1));
        }
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
        if (scenes.size() == 1) {   // run()'s frame slots, made here so that run() only copies
            const size_t slot = frame_floats + (size_t)std::max(n_rec, 1);
            const size_t total = slot * run_slot_count(slot);
            if (total * sizeof(float) <= (size_t(128) << 20)) reserve_run_slots(total);
        }

        // ---- tables and the job plan (autotuned, or from the plan cache), then the launch form
        for (size_t i = 0; i < buckets.size(); i++) {
            cudaStream_t s;
            CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            side.push_back(s);
        }
        // the cache serves unforced plans only (PSTD_MERGED / PSTD_PLAN / PSTD_DFT pin choices)
        const bool cacheable = autotune && !std::getenv("PSTD_MERGED") && !std::getenv("PSTD_PLAN") && !want_bf16_dft();
        const std::string sig = cacheable ? plan_signature() : std::string();
        PlanChoice cached;
        bool hit = false;
        if (cacheable) {
            std::lock_guard<std::mutex> lock(plan_cache_mutex());
            auto it = plan_cache().find(sig);
            if (it != plan_cache().end()) { cached = it->second; hit = true; }
        }
        reset();
        if (hit) {
            for (auto& b : buckets)
                for (auto& lv : cached.vars)
                    if (lv.first == b.L) { b.var = lv.second; b.choice = " (plan cache)"; }
            plan(false);
            longest_first = cached.longest_first;
            if (cached.merged) {
                merged_fam = cached.merged_fam;
                build_merged();
                merged = true;
                capture_graphs();
            }
            form_choice = cached.form + " (plan cache)";
        } else {
            plan(autotune);
            reset();
            if (autotune) {
                refine_plan();
                reset();
            }
            choose_form(autotune);
            if (cacheable) {
                PlanChoice pc;
                for (auto& b : buckets) pc.vars.push_back({b.L, b.var});
                pc.longest_first = longest_first;
                pc.merged = merged;
                pc.merged_fam = merged_fam;
                pc.form = form_choice;
                std::lock_guard<std::mutex> lock(plan_cache_mutex());
                plan_cache()[sig] = pc;
            }
        }
        if (!merged) capture_graphs();
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
        a.maps = dmaps.p;
        a.set_in = k == 0 ? c : ((k - 1) % 2 == 0 ? A : B);
        a.set_prev = c;
        a.err = derr.p;
        if (dev_counts) {
            a.scene_step = srv.scene_step;
            a.scene_limit = srv.limit;
        }
        return a;
    }

    // Tensor maps of the staged form: for every non-rigid domain the 2-D
    // [rows x columns] view of px, py, vx, vy in each state set and of its p0
    // array, boxes of 4 columns x tma_box_rows(rows) rows (stage_tma.cuh).
    // Needs the driver's cuTensorMapEncodeTiled; without it the staged
    // variants are left out of the plan.
    void build_tensor_maps() {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return;
        }
        auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        std::vector<unsigned char> maps((size_t)gdom.size() * 16 * PSTD_TMAP_BYTES, 0);
        auto put = [&](size_t idx, const float* base, int cols, int rows, int pitch) {
            CUtensorMap* m = reinterpret_cast<CUtensorMap*>(maps.data() + idx * PSTD_TMAP_BYTES);
            const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
            const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
            const cuuint32_t box[2] = {4, (cuuint32_t)tma_box_rows(rows)};
            const cuuint32_t estr[2] = {1, 1};
            const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                                      estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) throw CudaError("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        };
        for (size_t d = 0; d < gdom.size(); d++) {
            const DevDomain& h = hdoms[d];
            if (h.fixed) continue;
            for (int set = 0; set < 3; set++) {
                const float* b = sets[set].p;
                put((d * 4 + 0) * 4 + set, b + h.o_px, h.nx, h.ny, h.pitch_p);
                put((d * 4 + 1) * 4 + set, b + h.o_py, h.nx, h.ny, h.pitch_p);
                put((d * 4 + 2) * 4 + set, b + h.o_vx, h.nx + 1, h.ny, h.pitch_vx);
                put((d * 4 + 3) * 4 + set, b + h.o_vy, h.nx, h.ny + 1, h.pitch_vy);
            }
            put((d * 4 + 0) * 4 + 3, p0.p + h.o_p0, h.nx, h.ny, h.pitch_p);
        }
        dmaps.upload(maps);
    }

    // a device error word (a bounded wait that gave up, a job outside a form's
    // tile) is reported once, here
    void check_stage_error() {
        if (!derr.p) return;
        int e = 0;
        CK(cudaMemcpy(&e, derr.p, sizeof e, cudaMemcpyDeviceToHost));
        if (e) {
            CK(cudaMemset(derr.p, 0, sizeof(int)));
            throw CudaError(e == 3 ? "a stage-kernel job lies outside its form's fixed tile (error 3)"
                                   : "a bounded wait of the stage kernel (TMA copy or tensor-core commit) gave up "
                                     "(error " + std::to_string(e) + ")");
        }
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
    // tune_only (optional): tune just the buckets flagged there, keep the rest
    void plan(bool tune, const std::vector<bool>* tune_only = nullptr) {
        if (tune) {
            for (size_t bi = 0; bi < buckets.size(); bi++) {
                auto& b = buckets[bi];
                if (tune_only && !(*tune_only)[bi]) continue;
                if (b.pinned) continue;   // chosen by PSTD_PLAN or the precision study, not tuned
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
                    if (vs[i].bf16) all[i].clear();                                  // different arithmetic
                    if (vs[i].tma && !dmaps.p) all[i].clear();                       // no tensor maps here
                }
                upload_tables();
                float best = 1e30f;
                int best_i = 0;
                std::string rec;
                std::vector<std::pair<float, int>> timed;
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
                    // best of three trials of five launches (variants often differ by a
                    // few percent; one trial lets noise pick)
                    const int reps = 5;
                    float ms = 1e30f;
                    for (int trial = 0; trial < 3; trial++) {
                        CK(cudaEventRecord(e0, stream));
                        for (int w = 0; w < reps; w++) CK(vs[i].launch((int)all[i].size(), a, stream));
                        CK(cudaEventRecord(e1, stream));
                        CK(cudaEventSynchronize(e1));
                        float t;
                        CK(cudaEventElapsedTime(&t, e0, e1));
                        ms = std::min(ms, t / reps);
                    }
                    char buf[64];
                    std::snprintf(buf, sizeof buf, " %d:%.1fus", i, ms * 1e3f);
                    rec += buf;
                    if (ms < best) { best = ms; best_i = i; }
                    timed.push_back({ms, i});
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                b.var = &vs[best_i];
                b.choice = " tuned" + rec;
                std::sort(timed.begin(), timed.end());
                b.cands.clear();
                for (size_t q = 0; q < timed.size() && q < 8; q++) b.cands.push_back(&vs[timed[q].second]);
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

    int launches_per_step() const { return 6 * (int)stage_launches().size() + (n_pml > 0 || dev_counts) + 1; }

    // ---------------------------------------------------------------- merged form
    // One persistent launch per RK stage over the jobs of every length the
    // merged kernel supports (stage_all.cu); other lengths keep their own
    // launch.  Chosen at create time when it is faster on the scene's own steps.
    struct StageLaunch {
        const StageVariant* var;
        const DevJob* jobs;
        int n, tw_off, fp, fv, rc;
        bool all;
        const int* cnt = nullptr;   // device-count persistent launch (launch_dev): its job count
        int ctr = 0;                // and its job counter (counters[stage * 16 + ctr])
    };
    // serving form, one persistent launch per strip length: the configuration,
    // first job in djobs_all, index of the job count in dev_counts, twiddles
    struct DevRegion {
        const StageVariant* var;
        size_t base;
        int count_idx;
        int tw_off;
    };
    std::vector<DevRegion> dev_regions;
    struct SepBucket { int b, off, n; };
    bool merged = false;
    int merged_fam = merged_family_default();   // configuration family of the merged launch
    bool longest_first = false;   // launch order of the lengths in a stage (buckets ascend in L)
    DevBuf<DevJob> djobs_all, djobs_sep;
    int n_all = 0;
    std::vector<SepBucket> sep;
    DevBuf<int> counters;
    std::string form_choice;
    // serving form: counts in device memory, read by the launches themselves
    // ({long jobs, short jobs, offset of the short-job table, PML domains, PML
    // blocks, receivers, slots}); the tables behind them change in place
    // between steps
    const int* dev_counts = nullptr;

    std::vector<StageLaunch> stage_launches() const {
        std::vector<StageLaunch> v;
        if (dev_counts && !dev_regions.empty()) {
            for (size_t r = 0; r < dev_regions.size(); r++) {
                const DevRegion& g = dev_regions[r];
                StageLaunch l{g.var, djobs_all.p + g.base, 0, g.tw_off, 0, 0, 0, false};
                l.cnt = dev_counts + g.count_idx;
                l.ctr = (int)r;
                v.push_back(l);
            }
        } else if (merged) {
            if (n_all > 0 || dev_counts) v.push_back({nullptr, djobs_all.p, n_all, 0, 0, 0, 0, true});
            for (const SepBucket& q : sep) {
                const Bucket& b = buckets[q.b];
                v.push_back({b.var, djobs_sep.p + q.off, q.n, b.tw_off, b.fp_off, b.fv_off, b.rc, false});
            }
        } else {
            for (const Bucket& b : buckets) v.push_back({b.var, djobs.p + b.off, b.n, b.tw_off, b.fp_off, b.fv_off, b.rc, false});
            if (longest_first) std::reverse(v.begin(), v.end());
        }
        return v;
    }

    bool any_mergeable() const {
        for (const Bucket& b : buckets)
            if (merged_supports(b.L) && !b.pinned) return true;
        return false;
    }

    // job lists of the merged form: supported lengths (longest first, then the
    // copy jobs) in one list, the other lengths per bucket
    void build_merged() {
        std::vector<DevJob> all, rest;
        sep.clear();
        std::vector<int> order;
        for (size_t i = 0; i < buckets.size(); i++) order.push_back((int)i);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return buckets[a].L > buckets[b].L; });
        for (int i : order) {
            const Bucket& b = buckets[i];
            if (merged_supports(b.L) && !b.pinned) {
                auto js = make_jobs(b.L, merged_variant(b.L, merged_fam), false);
                all.insert(all.end(), js.begin(), js.end());
            } else {
                auto js = make_jobs(b.L, b.var, false);
                sep.push_back({i, (int)rest.size(), (int)js.size()});
                rest.insert(rest.end(), js.begin(), js.end());
            }
        }
        auto copies = make_jobs(-1, merged_variant(128, merged_fam), true);   // no strips of length -1: the copy jobs only
        all.insert(all.end(), copies.begin(), copies.end());
        n_all = (int)all.size();
        djobs_all.upload(all);
        djobs_sep.upload(rest);
        counters.alloc(6);
        CK(prepare_stage_all(merged_fam));
        upload_tables();
        while (side.size() < sep.size() + 1) {
            cudaStream_t st;
            CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            side.push_back(st);
        }
    }

    // device time of n steps replayed from the captured graphs (state advances)
    float time_steps(int n) {
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        for (int i = 0; i < 2; i++) step(stream);
        CK(cudaEventRecord(e0, stream));
        for (int i = 0; i < n; i++) step(stream);
        CK(cudaEventRecord(e1, stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return ms / n;
    }

    // the strip-job structure of the scenes (domain sizes and kinds, every strip
    // run with its neighbours and transform length): equal signatures get
    // equal job lists for every variant
    std::string plan_signature() const {
        std::string s;
        auto put = [&](long long v) { s += std::to_string(v); s += ','; };
        for (const Scene& sc : scenes) {
            put((long long)sc.doms.size());
            for (const Domain& d : sc.doms) { put(d.nx); put(d.ny); put(d.rigid); put(d.pml); put(d.update[0]); put(d.update[1]); }
            for (const StripRun& r : sc.runs) {
                put(r.dom); put(r.axis); put(r.first); put(r.count); put(r.d1); put(r.d2); put(run_length(sc, r));
            }
            s += ';';
        }
        return s;
    }

    // The isolated timing of plan() ranks each length alone, but a step runs
    // all lengths concurrently: one pass of coordinate descent over each
    // length's three fastest variants, timed on whole captured steps (the
    // state advances; the caller resets it).
    void refine_plan() {
        std::vector<size_t> order;
        for (size_t i = 0; i < buckets.size(); i++)
            if (buckets[i].cands.size() > 1) order.push_back(i);
        if (order.empty()) return;
        plan(false);
        capture_graphs();
        float best = time_steps(4);
        for (size_t i : order) {
            Bucket& b = buckets[i];
            const StageVariant* keep = b.var;
            for (const StageVariant* v : b.cands) {
                if (v == keep) continue;
                b.var = v;
                plan(false);
                capture_graphs();
                const float t = time_steps(4);
                if (t < best) { best = t; keep = v; }
            }
            if (b.var != keep) {
                b.var = keep;
                plan(false);
            }
            if (b.var != b.cands[0]) b.choice += std::string(" refined on whole steps: ") + b.var->name;
        }
        // launch order: longest transforms first or last (their CTAs run longest)
        longest_first = true;
        capture_graphs();
        if (time_steps(4) >= best) longest_first = false;
        capture_graphs();
    }

    // per-length launches vs the merged launch: keep the faster (PSTD_MERGED=0/1 forces)
    void choose_form(bool tune) {
        int force = -1;
        if (const char* e = std::getenv("PSTD_MERGED")) force = std::atoi(e) != 0;
        if (!any_mergeable() || force == 0 || (force < 0 && !tune)) {
            merged = false;
            form_choice = "per-length launches";
            return;
        }
        if (force == 1) {
            build_merged();
            merged = true;
            capture_graphs();
            form_choice = "merged launch (forced), family " + std::to_string(merged_fam);
            return;
        }
        merged = false;
        capture_graphs();
        const float t_len = time_steps(5);
        reset();
        // both configuration families of the merged launch (PSTD_MERGED_FAMILY: that one only)
        std::vector<int> fams{0, 1};
        if (std::getenv("PSTD_MERGED_FAMILY")) fams.assign(1, merged_family_default());
        float t_all = 1e30f;
        int best_fam = fams[0];
        std::string rec;
        for (int f : fams) {
            merged_fam = f;
            build_merged();
            merged = true;
            capture_graphs();
            const float t = time_steps(5);
            reset();
            char b[64];
            std::snprintf(b, sizeof b, "%s%.1f us family %d", rec.empty() ? "" : ", ", t * 1e3f, f);
            rec += b;
            if (t < t_all) { t_all = t; best_fam = f; }
        }
        char buf[200];
        std::snprintf(buf, sizeof buf, " (step merged %s vs %.1f us per length)", rec.c_str(), t_len * 1e3f);
        if (t_all >= t_len) {
            merged = false;
            capture_graphs();
            form_choice = std::string("per-length launches") + buf;
        } else {
            if (merged_fam != best_fam) {
                merged_fam = best_fam;
                build_merged();
                capture_graphs();
            }
            form_choice = std::string("merged launch, family ") + std::to_string(best_fam) + buf;
        }
    }

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
        if (merged) CK(cudaMemsetAsync(counters.p, 0, counters.n * sizeof(int), st));   // per-stage job counters
        for (int k = 0; k < 6; k++) {
            cudaEvent_t t0 = nullptr, t1 = nullptr;
            if (ev) {
                CK(cudaEventCreate(&t0));
                CK(cudaEventCreate(&t1));
                CK(cudaEventRecord(t0, st));
            }
            const std::vector<StageLaunch> ls = stage_launches();
            auto launch = [&](const StageLaunch& l, cudaStream_t s) {
                if (l.cnt) {
                    StageArgs a = stage_args(c, k, l.jobs, dtw.p + l.tw_off, 0, 0, 0);
                    CK(l.var->launch_dev(l.cnt, a, counters.p + k * 16 + l.ctr, s));
                } else if (l.all && dev_counts) {
                    CK(launch_stage_all_dev(merged_fam, dev_counts, stage_args(c, k, l.jobs, dtw.p, 0, 0, 0),
                                            counters.p + k, s));
                } else if (l.all) {
                    CK(launch_stage_all(merged_fam, l.n, stage_args(c, k, l.jobs, dtw.p, 0, 0, 0), counters.p + k, s));
                } else {
                    StageArgs a = stage_args(c, k, l.jobs, dtw.p + l.tw_off, l.fp, l.fv, l.rc);
                    CK(l.var->launch(l.n, a, s));
                }
            };
            if (concurrent && ls.size() > 1) {
                cudaEvent_t fork = mk();
                CK(cudaEventRecord(fork, st));
                std::vector<cudaEvent_t> joins;
                for (size_t i = 0; i < ls.size(); i++) {
                    cudaStream_t s = i == 0 ? st : side[i];
                    if (i > 0) CK(cudaStreamWaitEvent(s, fork, 0));
                    launch(ls[i], s);
                    if (i > 0) {
                        cudaEvent_t j = mk();
                        CK(cudaEventRecord(j, s));
                        joins.push_back(j);
                    }
                }
                for (auto j : joins) CK(cudaStreamWaitEvent(st, j, 0));
            } else {
                for (auto& l : ls) launch(l, st);
            }
            if (ev) {
                CK(cudaEventRecord(t1, st));
                ev->push_back({t0, t1});
            }
        }
        if (dev_counts)
            CK(launch_pml_post_dev(dpml.p, dev_counts + 3, dpml_off.p, ddoms.p, sets[B].p, fixed.p, p0.p, datt.p,
                                   srv.scene_step, srv.limit, st));
        else if (n_pml > 0)
            CK(launch_pml_post(dpml.p, n_pml, pml_blocks, ddoms.p, sets[B].p, fixed.p, p0.p, datt.p, st, dpml_off.p));
        if (srv.on) {
            CK(cudaMemsetAsync(first_step.p, 0, srv.n_flags * sizeof(int), st));
            CK(launch_server_receivers(srv.rec, n_rec, ddoms.p, sets[B].p, srv.aux, srv.scene_step, srv.limit,
                                       srv.slots, srv.n_slots, st, dev_counts ? dev_counts + 5 : nullptr));
        } else {
            CK(cudaMemsetAsync(first_step.p, 0, scenes.size() * sizeof(int), st));
            if (spectral)
                CK(launch_spectral_receivers(dsi_rows.p, n_si_rows, dsi_w.p, dsi_first.p, n_rec, ddoms.p, sets[B].p,
                                             fixed.p, p0.p, dsi_val.p, dring.p, ring_cap, dcounter.p, st));
            else
                CK(launch_receivers(drec.p, n_rec, ddoms.p, sets[B].p, dring.p, ring_cap, dcounter.p, st));
        }
        for (auto e : tmp) cudaEventDestroy(e);   // destruction is deferred until the event completes
    }

    void capture_graphs() {
        for (auto& g : graphs)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
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

}  // namespace pstd
