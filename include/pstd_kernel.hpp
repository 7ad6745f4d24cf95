// pstd_kernel.hpp -- openPSTD's C++ kernel API on the GB300 solver.
//
// Mirrors the classes of kernel/KernelInterface.h and kernel/PSTDKernel.h of
// the openPSTD tree (same names, members and semantics) in namespace
// pstd_gb300, with Qt's QVector2D / QVector3D replaced by plain structs.
// GpuPSTDKernel implements KernelInterface on top of the C ABI of
// pstd_gb300.h: it is the GPU branch of PSTDKernel::run
// (kernel/PSTDKernel.cpp:126-141) as a self-contained class.
//
// Errors follow the reference: run() / get_metadata() before
// initialize_kernel() throw PSTDKernelNotConfiguredException
// (kernel/PSTDKernel.cpp:122-123,155-156); failures of the GPU solve throw
// PSTDError carrying the C ABI status code and message.  An exception thrown
// by a callback stops the run at the next frame and is rethrown from run().
#pragma once

#include <cstdint>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pstd_gb300.h"

namespace pstd_gb300 {

// kernel/GeneralTypes.h:42-48
using PSTD_FRAME_UNIT = float;
using PSTD_FRAME = std::vector<PSTD_FRAME_UNIT>;
using PSTD_FRAME_PTR = std::shared_ptr<PSTD_FRAME>;

struct Vec2 {
    float v[2] = {0, 0};
    Vec2() = default;
    Vec2(float x, float y) { v[0] = x; v[1] = y; }
    float x() const { return v[0]; }
    float y() const { return v[1]; }
    float operator[](int i) const { return v[i]; }
};

struct Vec3 {
    float v[3] = {0, 0, 0};
    Vec3() = default;
    Vec3(float x, float y, float z) { v[0] = x; v[1] = y; v[2] = z; }
    float x() const { return v[0]; }
    float y() const { return v[1]; }
    float z() const { return v[2]; }
    float operator[](int i) const { return v[i]; }
};

// PSTD_DOMAIN_SIDE (kernel/KernelInterface.h:29-36)
enum PSTD_DOMAIN_SIDE {
    PSTD_DOMAIN_SIDE_TOP = 1,
    PSTD_DOMAIN_SIDE_BOTTOM = 2,
    PSTD_DOMAIN_SIDE_LEFT = 4,
    PSTD_DOMAIN_SIDE_RIGHT = 8,
    PSTD_DOMAIN_SIDE_ALL = 15,
    PSTD_DOMAIN_SIDE_NONE = 0
};

// kernel/KernelInterface.h:44-158
class PSTDSettings {
public:
    float calctime = 0, c1 = 0, ampMax = 0, freqMax = 0, rho = 0, patcherror = 0, tfactRK = 0, gridSpacing = 0,
          band_width = 0, wave_length = 0;
    std::vector<float> rk_coefficients;
    bool spectral_interpolation = false;
    bool spectral_receivers = false;   // PSTD_RECEIVERS_SPECTRAL (no reference counterpart; not in scene files)
    int PMLCells = 0;
    int SaveNth = 1;

    float GetGridSpacing() const { return gridSpacing; }
    void SetGridSpacing(float v) { gridSpacing = v; }
    float GetPatchError() const { return patcherror; }
    void SetPatchError(float v) { patcherror = v; }
    int GetWindowSize() const;
    float GetRenderTime() const { return calctime; }
    void SetRenderTime(float v) { calctime = v; }
    int GetPMLCells() const { return PMLCells; }
    void SetPMLCells(int v) { PMLCells = v; }
    float GetAttenuationOfPMLCells() const { return ampMax; }
    void SetAttenuationOfPMLCells(float v) { ampMax = v; }
    float GetDensityOfAir() const { return rho; }
    void SetDensityOfAir(float v) { rho = v; }
    float GetMaxFrequency() const { return freqMax; }
    void SetMaxFrequency(float v) { freqMax = v; }
    float GetSoundSpeed() const { return c1; }
    void SetSoundSpeed(float v) { c1 = v; }
    float GetFactRK() const { return tfactRK; }
    void SetFactRK(float v) { tfactRK = v; }
    int GetSaveNth() const { return SaveNth; }
    void SetSaveNth(int v) { SaveNth = v; }
    float GetBandWidth() const { return band_width; }
    void SetBandWidth(float v) { band_width = v; }
    bool GetSpectralInterpolation() const { return spectral_interpolation; }
    void SetSpectralInterpolation(bool v) { spectral_interpolation = v; }
    bool GetSpectralReceivers() const { return spectral_receivers; }
    void SetSpectralReceivers(bool v) { spectral_receivers = v; }
    float GetWaveLength() const { return wave_length; }
    void SetWaveLength(float v) { wave_length = v; }
    float GetTimeStep() const { return tfactRK * gridSpacing / c1; }
    std::vector<float> GetRKCoefficients() const { return rk_coefficients; }
    void SetRKCoefficients(std::vector<float> c) { rk_coefficients = std::move(c); }
};

// kernel/KernelInterface.h:163-175
class DomainConfEdge {
public:
    float Absorption = 0;
    bool LR = false;
};

// kernel/KernelInterface.h:180-205
class DomainConf {
public:
    Vec2 TopLeft, Size;
    DomainConfEdge T, L, B, R;
    float GetAbsorption(PSTD_DOMAIN_SIDE side) const;
    void SetAbsorption(PSTD_DOMAIN_SIDE sides, float absorption);
    bool GetLR(PSTD_DOMAIN_SIDE side) const;
    void SetLR(PSTD_DOMAIN_SIDE sides, bool LR);
};

// kernel/KernelInterface.h:213-240
class PSTDConfiguration {
public:
    PSTDSettings Settings;
    std::vector<Vec3> Speakers;
    std::vector<Vec3> Receivers;
    std::vector<DomainConf> Domains;
    static std::shared_ptr<PSTDConfiguration> CreateDefaultConf();   // kernel/KernelInterface.cpp:196-249
    static std::shared_ptr<PSTDConfiguration> CreateEmptyConf();
};

enum CALLBACKSTATUS { STARTING, RUNNING, FINISHED, ERROR };

// kernel/KernelInterface.h:243-271
class KernelCallbackLog {
public:
    virtual ~KernelCallbackLog() = default;
    virtual void Fatal(std::string message) {}
    virtual void Error(std::string message) {}
    virtual void Warning(std::string message) {}
    virtual void Info(std::string message) {}
    virtual void Debug(std::string message) {}
};

// kernel/KernelInterface.h:279-304
class KernelCallback : public KernelCallbackLog {
public:
    virtual void Callback(CALLBACKSTATUS status, std::string message, int frame) {}
    virtual void WriteFrame(int frame, int domain, PSTD_FRAME_PTR data) = 0;
    virtual void WriteSample(int startSample, int receiver, std::vector<float> data) = 0;
};

// kernel/KernelInterface.h:309-329
class SimulationMetadata {
public:
    std::vector<std::vector<int>> DomainMetadata;
    int Framecount = 0;
    std::vector<std::vector<int>> DomainPositions;
};

// kernel/KernelInterface.h:332-351
class KernelInterface {
public:
    virtual ~KernelInterface() = default;
    virtual void initialize_kernel(std::shared_ptr<PSTDConfiguration> config,
                                   std::shared_ptr<KernelCallbackLog> callbackLog) = 0;
    virtual void run(std::shared_ptr<KernelCallback> callback) = 0;
    virtual SimulationMetadata get_metadata() = 0;
};

class PSTDKernelNotConfiguredException : public std::exception {
public:
    const char* what() const noexcept override { return "The kernel is not yet configured"; }
};

class PSTDError : public std::runtime_error {
public:
    int code;
    PSTDError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// The GPU solver behind KernelInterface.
class GpuPSTDKernel : public KernelInterface {
public:
    GpuPSTDKernel() = default;
    ~GpuPSTDKernel() override;
    GpuPSTDKernel(const GpuPSTDKernel&) = delete;
    GpuPSTDKernel& operator=(const GpuPSTDKernel&) = delete;

    void initialize_kernel(std::shared_ptr<PSTDConfiguration> config,
                           std::shared_ptr<KernelCallbackLog> callbackLog) override;
    void run(std::shared_ptr<KernelCallback> callback) override;
    SimulationMetadata get_metadata() override;

    // device-resident extras (no reference counterpart)
    void advance(int n_steps);
    std::vector<float> receivers(int first_step, int n_steps);
    pstd_kernel* handle() const { return h_; }

private:
    pstd_kernel* h_ = nullptr;
    std::shared_ptr<PSTDConfiguration> config_;
    std::shared_ptr<KernelCallbackLog> log_;
};

// Pack a configuration into the C ABI struct; `storage` owns the arrays.
struct ConfigStorage {
    std::vector<pstd_domain_conf> domains;
    std::vector<float> speakers, receivers;
    pstd_config c{};
};
void to_c_config(const PSTDConfiguration& conf, ConfigStorage& storage);
std::shared_ptr<PSTDConfiguration> from_c_config(const pstd_config& c);

// shared/PSTDFile.h:134-159
class PSTDFileVersionException : public std::runtime_error {
public:
    explicit PSTDFileVersionException(const std::string& m) : std::runtime_error(m) {}
};
class PSTDFileIOException : public std::runtime_error {
public:
    int code;
    PSTDFileIOException(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Scene file (.pstd) with the results of runs: shared/PSTDFile.h:161-415 on
// the pstd_file_* C ABI.  unqlite_lib: the unqlite shared library ("" =
// $PSTD_UNQLITE_LIB, else libunqlite.so).
class PSTDFile {
public:
    static std::unique_ptr<PSTDFile> Open(const std::string& path, const std::string& unqlite_lib = "");
    static std::unique_ptr<PSTDFile> New(const std::string& path, const std::string& unqlite_lib = "");
    ~PSTDFile();
    PSTDFile(const PSTDFile&) = delete;
    PSTDFile& operator=(const PSTDFile&) = delete;

    void Commit();
    void Rollback();
    std::shared_ptr<PSTDConfiguration> GetSceneConf();
    void SetSceneConf(std::shared_ptr<PSTDConfiguration> scene);
    void InitializeResults();
    std::shared_ptr<PSTDConfiguration> GetResultsSceneConf();
    int GetResultsDomainCount();
    int GetResultsFrameCount(unsigned int domain);
    PSTD_FRAME_PTR GetResultsFrame(unsigned int frame, unsigned int domain);
    void SaveNextResultsFrame(unsigned int domain, PSTD_FRAME_PTR frame);
    void DeleteResults();
    void SaveReceiverData(unsigned int receiver, std::shared_ptr<std::vector<float>> data);
    std::shared_ptr<std::vector<float>> GetReceiverData(unsigned int receiver);
    int GetResultsReceiverCount();

private:
    explicit PSTDFile(pstd_file* h) : h_(h) {}
    pstd_file* h_ = nullptr;
};

}  // namespace pstd_gb300
