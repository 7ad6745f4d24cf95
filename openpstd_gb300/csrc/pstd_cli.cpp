// pstd_cli.cpp -- openPSTD's command line (CLI/main.cpp) on this library:
//
//   pstd-cli create <scene.pstd>
//   pstd-cli run [-f] <scene.pstd> [-g] [-m] [-M] [--debug]
//
// `create` writes a new scene file (PSTDFile::New: the default scene).
// `run` is RunCommand::execute (CLI/main.cpp:365-464): open the file, take
// its scene, delete old results, initialise new ones, run the kernel with an
// output that stores every frame and receiver sample in the file (CLIOutput,
// CLI/output.cpp:30-68), commit.  -g runs the GB300 solver (GpuPSTDKernel);
// this build has no CPU solver, so a run without -g (or with -m alone) is an
// error.  -M runs a stand-in kernel that computes nothing (frame f of every
// domain is Nx*Ny copies of f, receiver r gets f + r) -- like the
// reference's -M, for trying the file plumbing without a GPU.
//
// The scene file's key/value store (unqlite) is loaded from $PSTD_UNQLITE_LIB
// (else libunqlite.so).
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pstd_kernel.hpp"

using namespace pstd_gb300;

namespace {

// CLIOutput (CLI/output.cpp:30-68)
class CLIOutput : public KernelCallback {
public:
    CLIOutput(std::shared_ptr<PSTDFile> file, bool debug) : file_(std::move(file)), debug_(debug) {}
    void WriteFrame(int frame, int domain, PSTD_FRAME_PTR data) override {
        (void)frame;
        file_->SaveNextResultsFrame((unsigned)domain, data);
    }
    void WriteSample(int startSample, int receiver, std::vector<float> data) override {
        (void)startSample;
        file_->SaveReceiverData((unsigned)receiver, std::make_shared<std::vector<float>>(std::move(data)));
    }
    void Fatal(std::string m) override { std::cerr << "FATAL: " << m << std::endl; }
    void Error(std::string m) override { std::cerr << "ERROR: " << m << std::endl; }
    void Warning(std::string m) override { std::cout << "WARNING: " << m << std::endl; }
    void Info(std::string m) override { std::cout << m << std::endl; }
    void Debug(std::string m) override {
        if (debug_) std::cout << "DEBUG: " << m << std::endl;
    }

private:
    std::shared_ptr<PSTDFile> file_;
    bool debug_;
};

// stand-in kernel for -M: no computation, frames of the scene's domain sizes
class StandInKernel : public KernelInterface {
public:
    void initialize_kernel(std::shared_ptr<PSTDConfiguration> config, std::shared_ptr<KernelCallbackLog>) override {
        conf_ = std::move(config);
    }
    SimulationMetadata get_metadata() override {
        if (!conf_) throw PSTDKernelNotConfiguredException();
        SimulationMetadata m;
        const float dx = conf_->Settings.GetGridSpacing();
        for (const DomainConf& d : conf_->Domains)
            m.DomainMetadata.push_back({(int)(d.Size[0] / dx), (int)(d.Size[1] / dx), 0});
        m.Framecount = (int)(conf_->Settings.GetRenderTime() / conf_->Settings.GetTimeStep());
        return m;
    }
    void run(std::shared_ptr<KernelCallback> cb) override {
        const SimulationMetadata m = get_metadata();
        cb->Info("Starting the stand-in kernel");
        for (int f = 0; f < m.Framecount; f++) {
            for (size_t d = 0; d < m.DomainMetadata.size(); d++) {
                const size_t n = (size_t)m.DomainMetadata[d][0] * (size_t)m.DomainMetadata[d][1];
                cb->WriteFrame(f, (int)d, std::make_shared<std::vector<float>>(n, (float)f));
            }
            for (size_t r = 0; r < conf_->Receivers.size(); r++) cb->WriteSample(f, (int)r, {(float)(f + r)});
        }
        cb->Info("Finished the stand-in kernel");
    }

private:
    std::shared_ptr<PSTDConfiguration> conf_;
};

int usage() {
    std::cerr << "usage: pstd-cli create <scene.pstd>\n"
                 "       pstd-cli run [-f] <scene.pstd> [-g] [-m] [-M] [--debug]\n";
    return 1;
}

int create(int argc, char** argv) {
    if (argc < 1) return usage();
    PSTDFile::New(argv[0]);
    std::cout << "wrote the default scene to " << argv[0] << std::endl;
    return 0;
}

int run(int argc, char** argv) {
    std::string scene;
    bool gpu = false, mcpu = false, mock = false, debug = false;
    for (int i = 0; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "-g" || a == "--gpu-accelerated") gpu = true;
        else if (a == "-m" || a == "--multithreaded") mcpu = true;
        else if (a == "-M" || a == "--mock") mock = true;
        else if (a == "--debug") debug = true;
        else if ((a == "-f" || a == "--scene-file") && i + 1 < argc) scene = argv[++i];
        else if (a == "-h" || a == "--help") return usage() == 0;
        else if (!a.empty() && a[0] != '-') scene = a;
        else return usage();
    }
    if (scene.empty()) {
        std::cerr << "scene file is required" << std::endl;
        return usage();
    }
    if (mock && (gpu || mcpu))
        std::cout << "warning: no multithreaded or gpu accelerated versions of the mock kernel, using normal version"
                  << std::endl;
    if (!mock && !gpu) {
        std::cerr << "error: this build provides the GPU solver only; run with -g (or -M)" << std::endl;
        return 1;
    }
    std::shared_ptr<PSTDFile> file = PSTDFile::Open(scene);
    std::shared_ptr<PSTDConfiguration> conf = file->GetSceneConf();
    std::cout << "Delete old results(if any)" << std::endl;
    file->DeleteResults();
    std::cout << "initilize new results" << std::endl;
    file->InitializeResults();
    std::unique_ptr<KernelInterface> kernel;
    if (mock) kernel.reset(new StandInKernel());
    else kernel.reset(new GpuPSTDKernel());
    auto output = std::make_shared<CLIOutput>(file, debug);
    kernel->initialize_kernel(conf, output);
    kernel->run(output);
    file->Commit();
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return usage();
    try {
        const std::string cmd = argv[1];
        if (cmd == "create") return create(argc - 2, argv + 2);
        if (cmd == "run") return run(argc - 2, argv + 2);
        return usage();
    } catch (std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
}
