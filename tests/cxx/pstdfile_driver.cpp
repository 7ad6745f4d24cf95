// Drives pstd_gb300::PSTDFile (include/pstd_kernel.hpp) the way the
// reference's CLI drives OpenPSTD::Shared::PSTDFile (CLI/main.cpp:419-449),
// and prints what it read back as JSON.  Usage: pstdfile_driver <file> <unqlite library>
#include <cstdio>
#include <string>

#include "pstd_kernel.hpp"

using namespace pstd_gb300;

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::string path = argv[1], lib = argv[2];
    {
        auto f = PSTDFile::New(path, lib);
        auto conf = f->GetSceneConf();             // CreateDefaultConf
        conf->Receivers.push_back(Vec3(7.5f, 6.5f, 0.f));
        f->SetSceneConf(conf);
        f->InitializeResults();
        for (int k = 0; k < 3; k++) f->SaveNextResultsFrame(1, std::make_shared<std::vector<float>>(4, 0.5f * k));
        f->SaveReceiverData(1, std::make_shared<std::vector<float>>(2, 1.25f));
        f->Commit();
    }
    auto g = PSTDFile::Open(path, lib);
    auto conf = g->GetSceneConf();
    bool version_error = false;
    try {
        PSTDFile::Open(path + ".missing", lib);
    } catch (PSTDFileIOException&) {
        version_error = true;   // not a PSTD file: no version record
    }
    auto frame = g->GetResultsFrame(2, 1);
    auto samples = g->GetReceiverData(1);
    std::printf("{\"domains\": %zu, \"receivers\": %zu, \"results_domains\": %d, \"frames\": %d, "
                "\"frame2\": %g, \"samples\": %zu, \"sample0\": %g, \"open_missing_throws\": %s, "
                "\"pml\": %d, \"window\": %d}\n",
                conf->Domains.size(), conf->Receivers.size(), g->GetResultsDomainCount(),
                g->GetResultsFrameCount(1), (*frame)[3], samples->size(), (*samples)[0],
                version_error ? "true" : "false", conf->Settings.GetPMLCells(), conf->Settings.GetWindowSize());
    return 0;
}
