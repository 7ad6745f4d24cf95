// Drives the C++ kernel API (include/pstd_kernel.hpp) the way openPSTD's CLI
// drives PSTDKernel (CLI/main.cpp:431-449): configure, query metadata, run
// with a callback that keeps frames and samples.  Prints one JSON line.
//   kernel_api_driver check       -- no GPU needed: API errors only
//   kernel_api_driver run N       -- square scene, N frames, receivers + checksums
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "pstd_kernel.hpp"

using namespace pstd_gb300;

struct Collect : KernelCallback {
    std::map<int, std::vector<float>> samples;
    int frames = 0;
    double frame_sum = 0;
    std::vector<std::string> info;
    bool keep = false;                      // keep every frame (big mode)
    std::vector<PSTD_FRAME_PTR> kept;
    std::vector<double> sums;               // per frame, at delivery
    void WriteFrame(int frame, int domain, PSTD_FRAME_PTR data) override {
        frames++;
        double s = 0;
        for (float v : *data) s += v;
        frame_sum += s;
        if (keep) {
            kept.push_back(data);
            sums.push_back(s);
        }
    }
    void WriteSample(int start, int receiver, std::vector<float> data) override {
        samples[receiver].insert(samples[receiver].end(), data.begin(), data.end());
    }
    void Info(std::string m) override { info.push_back(m); }
};

static std::shared_ptr<PSTDConfiguration> square(int frames) {
    auto conf = PSTDConfiguration::CreateDefaultConf();
    conf->Domains.clear();
    DomainConf d;
    d.TopLeft = Vec2(0, 0);
    d.Size = Vec2(12.f, 12.f);   // 60 x 60 cells at dx = 0.2
    d.SetAbsorption(PSTD_DOMAIN_SIDE_ALL, 1.f);
    conf->Domains.push_back(d);
    conf->Settings.SetPMLCells(40);
    conf->Speakers = {Vec3(5.05f, 6.05f, 0)};
    conf->Receivers = {Vec3(7.05f, 6.05f, 0), Vec3(3.05f, 8.05f, 0)};
    conf->Settings.SetRenderTime((frames + 0.5f) * conf->Settings.GetTimeStep());
    return conf;
}

int main(int argc, char** argv) {
    std::string mode = argc > 1 ? argv[1] : "check";
    if (mode == "check") {
        GpuPSTDKernel k;
        bool not_configured = false;
        try { k.get_metadata(); } catch (PSTDKernelNotConfiguredException&) { not_configured = true; }
        bool run_not_configured = false;
        try { k.run(std::make_shared<Collect>()); } catch (PSTDKernelNotConfiguredException&) { run_not_configured = true; }
        auto conf = PSTDConfiguration::CreateDefaultConf();
        ConfigStorage st;
        to_c_config(*conf, st);
        std::printf("{\"not_configured\": %s, \"run_not_configured\": %s, \"window\": %d, \"domains\": %d, \"dt\": %.9g}\n",
                    not_configured ? "true" : "false", run_not_configured ? "true" : "false",
                    conf->Settings.GetWindowSize(), st.c.n_domains, conf->Settings.GetTimeStep());
        return 0;
    }
    int frames = argc > 2 ? std::atoi(argv[2]) : 20;
    if (mode == "big") {
        // 1000 x 600 cells: frames large enough for the device to copy them
        // straight into pooled page-locked vectors; every frame is kept and
        // summed again after the run (a vector reused while held would differ)
        auto conf = square(frames);
        conf->Domains[0].Size = Vec2(200.f, 120.f);
        conf->Speakers = {Vec3(100.05f, 60.05f, 0)};
        conf->Receivers = {Vec3(30.05f, 20.05f, 0)};
        GpuPSTDKernel k;
        k.initialize_kernel(conf, std::make_shared<KernelCallbackLog>());
        auto cb = std::make_shared<Collect>();
        cb->keep = true;
        k.run(cb);
        std::printf("{\"frames\": %d, \"size\": %zu, \"sums\": [", cb->frames, cb->kept.empty() ? 0 : cb->kept[0]->size());
        for (size_t i = 0; i < cb->sums.size(); i++) std::printf("%s%.17g", i ? ", " : "", cb->sums[i]);
        std::printf("], \"resums\": [");
        for (size_t i = 0; i < cb->kept.size(); i++) {
            double r = 0;
            for (float v : *cb->kept[i]) r += v;
            std::printf("%s%.17g", i ? ", " : "", r);
        }
        std::printf("]}\n");
        return 0;
    }
    auto conf = square(frames);
    GpuPSTDKernel k;
    k.initialize_kernel(conf, std::make_shared<KernelCallbackLog>());
    SimulationMetadata md = k.get_metadata();
    auto cb = std::make_shared<Collect>();
    k.run(cb);
    std::printf("{\"framecount\": %d, \"n_domains\": %zu, \"frames\": %d, \"frame_sum\": %.9g, \"info\": %zu, \"receivers\": [",
                md.Framecount, md.DomainMetadata.size(), cb->frames, cb->frame_sum, cb->info.size());
    bool first = true;
    for (auto& kv : cb->samples) {
        std::printf("%s[", first ? "" : ", ");
        first = false;
        for (size_t i = 0; i < kv.second.size(); i++) std::printf("%s%.9g", i ? ", " : "", kv.second[i]);
        std::printf("]");
    }
    std::printf("]}\n");
    return 0;
}
