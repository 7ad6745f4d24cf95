// gpu_pstd_kernel.cpp -- the C++ kernel API (include/pstd_kernel.hpp) on
// the C ABI (include/pstd_gb300.h).
#include "../../include/pstd_kernel.hpp"

#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <map>

namespace pstd_gb300 {

int PSTDSettings::GetWindowSize() const {
    // kernel/KernelInterface.cpp:128-134
    int tmp = (int)std::round((patcherror * 0.7 - 17) / 2.);
    return (int)std::round(tmp * 2);
}

static const DomainConfEdge* edge_of(const DomainConf& d, PSTD_DOMAIN_SIDE s) {
    switch (s) {
        case PSTD_DOMAIN_SIDE_TOP: return &d.T;
        case PSTD_DOMAIN_SIDE_BOTTOM: return &d.B;
        case PSTD_DOMAIN_SIDE_LEFT: return &d.L;
        case PSTD_DOMAIN_SIDE_RIGHT: return &d.R;
        default: return nullptr;
    }
}

float DomainConf::GetAbsorption(PSTD_DOMAIN_SIDE side) const {
    const DomainConfEdge* e = edge_of(*this, side);
    return e ? e->Absorption : 0;
}

bool DomainConf::GetLR(PSTD_DOMAIN_SIDE side) const {
    const DomainConfEdge* e = edge_of(*this, side);
    return e ? e->LR : false;
}

void DomainConf::SetAbsorption(PSTD_DOMAIN_SIDE sides, float a) {
    if (sides & PSTD_DOMAIN_SIDE_TOP) T.Absorption = a;
    if (sides & PSTD_DOMAIN_SIDE_BOTTOM) B.Absorption = a;
    if (sides & PSTD_DOMAIN_SIDE_LEFT) L.Absorption = a;
    if (sides & PSTD_DOMAIN_SIDE_RIGHT) R.Absorption = a;
}

void DomainConf::SetLR(PSTD_DOMAIN_SIDE sides, bool lr) {
    if (sides & PSTD_DOMAIN_SIDE_TOP) T.LR = lr;
    if (sides & PSTD_DOMAIN_SIDE_BOTTOM) B.LR = lr;
    if (sides & PSTD_DOMAIN_SIDE_LEFT) L.LR = lr;
    if (sides & PSTD_DOMAIN_SIDE_RIGHT) R.LR = lr;
}

std::shared_ptr<PSTDConfiguration> PSTDConfiguration::CreateDefaultConf() {
    // kernel/KernelInterface.cpp:196-249
    auto conf = std::make_shared<PSTDConfiguration>();
    PSTDSettings& s = conf->Settings;
    s.SetRenderTime(1.0f);
    float sound_speed = 340, grid_spacing = 0.2f;
    s.SetSoundSpeed(sound_speed);
    s.SetAttenuationOfPMLCells(20000.0f);
    s.SetDensityOfAir(1.2f);
    s.SetPatchError(70.0f);
    s.SetFactRK(0.5f);
    s.SetGridSpacing(grid_spacing);
    s.SetPMLCells(50);
    s.SetSaveNth(1);
    s.SetBandWidth((float)(3 * 1e-6 * (sound_speed / grid_spacing) * (sound_speed / grid_spacing)));
    s.SetRKCoefficients({1.179799016570605e-1f, 1.846469664911166e-1f, 2.466236043095944e-1f,
                         3.318395427360000e-1f, 5e-1f, 1.f});
    s.SetSpectralInterpolation(true);
    conf->Speakers.push_back(Vec3(4, 5, 0));
    conf->Receivers.push_back(Vec3(6, 5, 0));
    DomainConf d, d2;
    d.TopLeft = Vec2(0, 0);
    d.Size = Vec2(10, 15);
    d.T.Absorption = 1; d.B.Absorption = 0; d.L.Absorption = .3f; d.R.Absorption = 1;
    d2.TopLeft = Vec2(10, 4);
    d2.Size = Vec2(20, 15);
    d2.T.Absorption = 1; d2.B.Absorption = 0; d2.L.Absorption = 1; d2.R.Absorption = 1;
    conf->Domains.push_back(d);
    conf->Domains.push_back(d2);
    return conf;
}

std::shared_ptr<PSTDConfiguration> PSTDConfiguration::CreateEmptyConf() {
    auto conf = std::make_shared<PSTDConfiguration>();
    conf->Settings.SetSaveNth(0);
    return conf;
}

void to_c_config(const PSTDConfiguration& conf, ConfigStorage& st) {
    const PSTDSettings& s = conf.Settings;
    pstd_settings& c = st.c.settings;
    std::memset(&c, 0, sizeof c);
    c.calctime = s.calctime; c.c1 = s.c1; c.ampMax = s.ampMax; c.freqMax = s.freqMax; c.rho = s.rho;
    c.patcherror = s.patcherror; c.tfactRK = s.tfactRK; c.gridSpacing = s.gridSpacing;
    c.band_width = s.band_width; c.wave_length = s.wave_length;
    c.n_rk_coefficients = (int32_t)s.rk_coefficients.size();
    for (size_t i = 0; i < s.rk_coefficients.size() && i < 6; i++) c.rk_coefficients[i] = s.rk_coefficients[i];
    c.spectral_interpolation = s.spectral_receivers ? PSTD_RECEIVERS_SPECTRAL : (int32_t)s.spectral_interpolation;
    c.PMLCells = s.PMLCells;
    c.SaveNth = s.SaveNth;
    st.domains.clear();
    for (const DomainConf& d : conf.Domains) {
        pstd_domain_conf x;
        x.top_left[0] = d.TopLeft[0]; x.top_left[1] = d.TopLeft[1];
        x.size[0] = d.Size[0]; x.size[1] = d.Size[1];
        x.T = {d.T.Absorption, d.T.LR}; x.L = {d.L.Absorption, d.L.LR};
        x.B = {d.B.Absorption, d.B.LR}; x.R = {d.R.Absorption, d.R.LR};
        st.domains.push_back(x);
    }
    st.speakers.clear();
    for (const Vec3& p : conf.Speakers) st.speakers.insert(st.speakers.end(), {p[0], p[1], p[2]});
    st.receivers.clear();
    for (const Vec3& p : conf.Receivers) st.receivers.insert(st.receivers.end(), {p[0], p[1], p[2]});
    st.c.n_domains = (int32_t)st.domains.size();
    st.c.domains = st.domains.data();
    st.c.n_speakers = (int32_t)conf.Speakers.size();
    st.c.speakers = st.speakers.data();
    st.c.n_receivers = (int32_t)conf.Receivers.size();
    st.c.receivers = st.receivers.data();
}

namespace {

void check(int rc) {
    if (rc != PSTD_OK) throw PSTDError(rc, pstd_last_error());
}

void log_bridge(void* user, int32_t level, const char* msg) {
    auto* log = static_cast<KernelCallbackLog*>(user);
    if (!log) return;
    try {
        switch (level) {
            case PSTD_LOG_FATAL: log->Fatal(msg); break;
            case PSTD_LOG_ERROR: log->Error(msg); break;
            case PSTD_LOG_WARNING: log->Warning(msg); break;
            case PSTD_LOG_INFO: log->Info(msg); break;
            default: log->Debug(msg); break;
        }
    } catch (...) {
        // logging is non-blocking and must not stop the kernel
    }
}

// Frame vectors handed to WriteFrame are recycled and page-locked: the
// device copies a frame straight into the vector the callee receives
// (pstd_callbacks.frame_buffer), and a fresh multi-megabyte vector would be
// faulted in and zeroed by the OS every time.  A vector returns to the pool
// when the callee drops its last reference (the shared_ptr's deleter), from
// any thread; the pool is never destroyed, so late deleters stay valid.
struct FramePool {
    std::mutex m;
    std::vector<PSTD_FRAME*> free;
    std::set<const float*> locked;   // data() of page-locked vectors
    static constexpr size_t KEEP = 32;
    static constexpr int64_t DIRECT_MIN = 1 << 19;   // floats: smaller frames are copied

    // a vector of n floats (contents unspecified), page-locked if `lock`
    PSTD_FRAME* take(int64_t n, bool lock) {
        PSTD_FRAME* v = nullptr;
        {
            std::lock_guard<std::mutex> g(m);
            for (size_t i = 0; i < free.size(); i++)
                if (free[i]->capacity() >= (size_t)n) {
                    v = free[i];
                    free.erase(free.begin() + (long)i);
                    break;
                }
        }
        if (!v) v = new PSTD_FRAME();
        v->resize((size_t)n);   // within capacity: data() does not move
        if (lock) {
            std::lock_guard<std::mutex> g(m);
            if (!locked.count(v->data()) && pstd_host_register(v->data(), (int64_t)(v->capacity() * sizeof(float))) == PSTD_OK)
                locked.insert(v->data());
        }
        return v;
    }
    bool is_locked(const float* p) {
        std::lock_guard<std::mutex> g(m);
        return locked.count(p) != 0;
    }
    PSTD_FRAME_PTR share(PSTD_FRAME* v) {
        return PSTD_FRAME_PTR(v, [this](PSTD_FRAME* q) { give(q); });
    }
    void give(PSTD_FRAME* q) {
        {
            std::lock_guard<std::mutex> g(m);
            if (free.size() < KEEP) {
                free.push_back(q);
                return;
            }
            if (locked.erase(q->data())) pstd_host_unregister(q->data());
        }
        delete q;
    }
};

FramePool& frame_pool() {
    static FramePool* pool = new FramePool();
    return *pool;
}

struct RunCtx {
    KernelCallback* cb;
    std::exception_ptr error;
    std::map<const float*, PSTD_FRAME*> inflight;   // frames the device copies into pooled vectors
};

float* frame_buffer_bridge(void* user, int32_t, int32_t, int64_t n) {
    auto* ctx = static_cast<RunCtx*>(user);
    if (n < FramePool::DIRECT_MIN) return nullptr;
    try {
        PSTD_FRAME* v = frame_pool().take(n, true);
        if (!frame_pool().is_locked(v->data())) {   // not page-locked: the library stages it
            frame_pool().give(v);
            return nullptr;
        }
        ctx->inflight[v->data()] = v;
        return v->data();
    } catch (...) {
        return nullptr;
    }
}

int frame_bridge(void* user, int32_t frame, int32_t domain, const float* data, int64_t n) {
    auto* ctx = static_cast<RunCtx*>(user);
    try {
        // the callee may keep the frame (kernel/KernelInterface.h:285-290)
        PSTD_FRAME_PTR f;
        auto it = ctx->inflight.find(data);
        if (it != ctx->inflight.end()) {   // the device copied it into a pooled vector: hand that over
            f = frame_pool().share(it->second);
            ctx->inflight.erase(it);
        } else {
            PSTD_FRAME* v = frame_pool().take(n, false);
            std::memcpy(v->data(), data, (size_t)n * sizeof(float));
            f = frame_pool().share(v);
        }
        ctx->cb->WriteFrame(frame, domain, f);
        return 0;
    } catch (...) {
        ctx->error = std::current_exception();
        return 1;
    }
}

int sample_bridge(void* user, int32_t start, int32_t receiver, const float* data, int64_t n) {
    auto* ctx = static_cast<RunCtx*>(user);
    try {
        ctx->cb->WriteSample(start, receiver, std::vector<float>(data, data + n));
        return 0;
    } catch (...) {
        ctx->error = std::current_exception();
        return 1;
    }
}

void run_log_bridge(void* user, int32_t level, const char* msg) {
    log_bridge(static_cast<RunCtx*>(user)->cb, level, msg);
}

}  // namespace

GpuPSTDKernel::~GpuPSTDKernel() { pstd_destroy(h_); }

void GpuPSTDKernel::initialize_kernel(std::shared_ptr<PSTDConfiguration> config,
                                      std::shared_ptr<KernelCallbackLog> callbackLog) {
    if (!config) throw PSTDError(PSTD_ERR_INVALID, "null configuration");
    pstd_destroy(h_);
    h_ = nullptr;
    config_ = config;
    log_ = callbackLog;
    ConfigStorage st;
    to_c_config(*config, st);
    pstd_callbacks cb{};
    cb.user = log_.get();
    cb.log = log_ ? &log_bridge : nullptr;
    check(pstd_create(&st.c, &cb, &h_));
}

void GpuPSTDKernel::run(std::shared_ptr<KernelCallback> callback) {
    if (!h_) throw PSTDKernelNotConfiguredException();
    RunCtx ctx{callback.get(), nullptr, {}};
    pstd_callbacks cb{};
    cb.user = &ctx;
    if (callback) {
        cb.write_frame = &frame_bridge;
        cb.write_sample = &sample_bridge;
        cb.log = &run_log_bridge;
        cb.frame_buffer = &frame_buffer_bridge;
    }
    int rc = pstd_run(h_, &cb);
    for (auto& kv : ctx.inflight) frame_pool().give(kv.second);   // frames a stopped run never delivered
    if (ctx.error) std::rethrow_exception(ctx.error);
    check(rc);
}

SimulationMetadata GpuPSTDKernel::get_metadata() {
    if (!h_) throw PSTDKernelNotConfiguredException();
    int32_t n = 0, fc = 0;
    check(pstd_get_metadata(h_, &n, nullptr, 0, &fc));
    std::vector<int32_t> dims(3 * (size_t)n);
    check(pstd_get_metadata(h_, &n, dims.data(), n, &fc));
    SimulationMetadata md;
    for (int i = 0; i < n; i++) md.DomainMetadata.push_back({dims[3 * i], dims[3 * i + 1], dims[3 * i + 2]});
    md.Framecount = fc;
    return md;
}

void GpuPSTDKernel::advance(int n_steps) {
    if (!h_) throw PSTDKernelNotConfiguredException();
    check(pstd_advance(h_, n_steps, nullptr));
    check(pstd_synchronize(h_));
}

std::vector<float> GpuPSTDKernel::receivers(int first_step, int n_steps) {
    if (!h_) throw PSTDKernelNotConfiguredException();
    std::vector<float> out((size_t)n_steps * config_->Receivers.size());
    check(pstd_get_receivers(h_, first_step, n_steps, out.data()));
    return out;
}

}  // namespace pstd_gb300

namespace pstd_gb300 {

std::shared_ptr<PSTDConfiguration> from_c_config(const pstd_config& c) {
    auto conf = std::make_shared<PSTDConfiguration>();
    PSTDSettings& s = conf->Settings;
    const pstd_settings& x = c.settings;
    s.calctime = x.calctime; s.c1 = x.c1; s.ampMax = x.ampMax; s.freqMax = x.freqMax; s.rho = x.rho;
    s.patcherror = x.patcherror; s.tfactRK = x.tfactRK; s.gridSpacing = x.gridSpacing;
    s.band_width = x.band_width; s.wave_length = x.wave_length;
    s.rk_coefficients.assign(x.rk_coefficients, x.rk_coefficients + (x.n_rk_coefficients > 6 ? 6 : x.n_rk_coefficients));
    s.spectral_interpolation = x.spectral_interpolation != 0;
    s.spectral_receivers = x.spectral_interpolation == PSTD_RECEIVERS_SPECTRAL;
    s.PMLCells = x.PMLCells;
    s.SaveNth = x.SaveNth;
    for (int i = 0; i < c.n_speakers; i++)
        conf->Speakers.push_back(Vec3(c.speakers[3 * i], c.speakers[3 * i + 1], c.speakers[3 * i + 2]));
    for (int i = 0; i < c.n_receivers; i++)
        conf->Receivers.push_back(Vec3(c.receivers[3 * i], c.receivers[3 * i + 1], c.receivers[3 * i + 2]));
    for (int i = 0; i < c.n_domains; i++) {
        const pstd_domain_conf& d = c.domains[i];
        DomainConf o;
        o.TopLeft = Vec2(d.top_left[0], d.top_left[1]);
        o.Size = Vec2(d.size[0], d.size[1]);
        o.T = {d.T.absorption, d.T.lr != 0};
        o.L = {d.L.absorption, d.L.lr != 0};
        o.B = {d.B.absorption, d.B.lr != 0};
        o.R = {d.R.absorption, d.R.lr != 0};
        conf->Domains.push_back(o);
    }
    return conf;
}

// status -> the reference's PSTDFile exceptions
static void file_check(int rc) {
    if (rc == PSTD_OK) return;
    const std::string m = pstd_file_last_error();
    if (rc == PSTD_ERR_UNSUPPORTED && m.rfind("Wrong version", 0) == 0) throw PSTDFileVersionException(m);
    throw PSTDFileIOException(rc, m);
}

std::unique_ptr<PSTDFile> PSTDFile::Open(const std::string& path, const std::string& lib) {
    pstd_file* h = nullptr;
    file_check(pstd_file_open(path.c_str(), lib.empty() ? nullptr : lib.c_str(), 0, &h));
    return std::unique_ptr<PSTDFile>(new PSTDFile(h));
}

std::unique_ptr<PSTDFile> PSTDFile::New(const std::string& path, const std::string& lib) {
    pstd_file* h = nullptr;
    file_check(pstd_file_open(path.c_str(), lib.empty() ? nullptr : lib.c_str(), 1, &h));
    return std::unique_ptr<PSTDFile>(new PSTDFile(h));
}

PSTDFile::~PSTDFile() { pstd_file_close(h_); }
void PSTDFile::Commit() { file_check(pstd_file_commit(h_)); }
void PSTDFile::Rollback() { file_check(pstd_file_rollback(h_)); }

std::shared_ptr<PSTDConfiguration> PSTDFile::GetSceneConf() {
    pstd_config c{};
    file_check(pstd_file_get_scene(h_, 0, &c));
    return from_c_config(c);
}

std::shared_ptr<PSTDConfiguration> PSTDFile::GetResultsSceneConf() {
    pstd_config c{};
    file_check(pstd_file_get_scene(h_, 1, &c));
    return from_c_config(c);
}

void PSTDFile::SetSceneConf(std::shared_ptr<PSTDConfiguration> scene) {
    ConfigStorage st;
    to_c_config(*scene, st);
    file_check(pstd_file_set_scene(h_, 0, &st.c));
}

void PSTDFile::InitializeResults() { file_check(pstd_file_initialize_results(h_)); }
void PSTDFile::DeleteResults() { file_check(pstd_file_delete_results(h_)); }
int PSTDFile::GetResultsDomainCount() { return (int)GetResultsSceneConf()->Domains.size(); }
int PSTDFile::GetResultsReceiverCount() { return (int)GetResultsSceneConf()->Receivers.size(); }

int PSTDFile::GetResultsFrameCount(unsigned int domain) {
    int32_t n = 0;
    file_check(pstd_file_frame_count(h_, (int32_t)domain, &n));
    return n;
}

PSTD_FRAME_PTR PSTDFile::GetResultsFrame(unsigned int frame, unsigned int domain) {
    int64_t n = 0;
    file_check(pstd_file_get_frame(h_, (int32_t)domain, (int32_t)frame, nullptr, 0, &n));
    auto out = std::make_shared<std::vector<float>>((size_t)n);
    file_check(pstd_file_get_frame(h_, (int32_t)domain, (int32_t)frame, out->data(), n, &n));
    return out;
}

void PSTDFile::SaveNextResultsFrame(unsigned int domain, PSTD_FRAME_PTR frame) {
    file_check(pstd_file_save_frame(h_, (int32_t)domain, frame->data(), (int64_t)frame->size()));
}

void PSTDFile::SaveReceiverData(unsigned int receiver, std::shared_ptr<std::vector<float>> data) {
    file_check(pstd_file_append_samples(h_, (int32_t)receiver, data->data(), (int64_t)data->size()));
}

std::shared_ptr<std::vector<float>> PSTDFile::GetReceiverData(unsigned int receiver) {
    int64_t n = 0;
    file_check(pstd_file_get_samples(h_, (int32_t)receiver, nullptr, 0, &n));
    auto out = std::make_shared<std::vector<float>>((size_t)n);
    file_check(pstd_file_get_samples(h_, (int32_t)receiver, out->data(), n, &n));
    return out;
}

}  // namespace pstd_gb300
