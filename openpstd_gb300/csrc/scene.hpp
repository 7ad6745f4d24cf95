// scene.hpp -- host-side scene model of the GB300 PSTD solve.
//
// Builds, from a pstd_config, the same scene the reference's PSTDKernel builds
// (kernel/PSTDKernel.cpp:62-119, kernel/core/Scene.cpp:41-380,
// kernel/core/Domain.cpp:53-92,504-780): air domains, automatic primary and
// corner PML domains, neighbour lists, update flags, PML attenuation profiles,
// speakers and receivers.  The result is flattened into the plan the device
// kernels consume: per-domain field layout and, per strip direction, a list of
// strip jobs (which neighbour supplies the interface band of every row or
// column, with its reflection/transmission coefficients).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pstd_gb300.h"

namespace pstd {

struct SceneError : std::runtime_error {
    int code;
    SceneError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum Side { S_LEFT = 0, S_RIGHT = 1, S_TOP = 2, S_BOTTOM = 3 };   // TOP = smaller y
enum Axis { AX_X = 0, AX_Y = 1 };

struct Settings {
    float calctime, c1, ampMax, rho, patcherror, tfactRK, dx, band_width;
    float rk[6];
    int pml_cells, save_nth;
    float dt() const;          // tfactRK*dx/c1 in float
    int window() const;        // window length from the patch error
    int framecount() const;    // (int)(calctime/dt)
};

struct Domain {
    int id = 0;
    int x0 = 0, y0 = 0, nx = 0, ny = 0;     // grid rectangle
    float alpha = 1.f;
    float impedance = 1.f, rho = 0.f;       // float, as the reference stores them
    bool pml = false, secondary = false, rigid = false, local = false;
    std::vector<int> parents;               // "pml_for" list (pool indices)
    float edge_alpha[4] = {0, 0, 0, 0};
    bool edge_lr[4] = {false, false, false, false};
    std::vector<int> nb[4];                 // neighbours per side (pool indices during build, scene indices after)
    bool update[2] = {true, true};
    // attenuation: which axes carry a profile and their orientation
    bool att_x = false, att_y = false, asc_x = false, asc_y = false;

    int x1() const { return x0 + nx; }
    int y1() const { return y0 + ny; }
    int lo(Axis a) const { return a == AX_X ? y0 : x0; }   // strip-index range of an axis pass
    int hi(Axis a) const { return a == AX_X ? y1() : x1(); }
    int len(Axis a) const { return a == AX_X ? nx : ny; }   // strip length (pressure cells)
};

struct Receiver {
    int id;
    int dom;          // scene index of the container
    int row, col;     // element of p0 the reference reads: p0(rel.x, rel.y) -> row rel.x, column rel.y
                      // (spectral receivers: x offset, y offset of the cell holding the point)
    float gx, gy;     // grid location (world / dx)
};

struct Speaker { float x, y; };   // grid coordinates after the -0.5 shift

// One run of consecutive strips of one domain that share both neighbours.
struct StripRun {
    int dom;
    Axis axis;
    int first, count;    // strips relative to the domain (rows for X, columns for Y)
    int d1, d2;          // neighbour scene indices on the low/high side or -1 (X: left/right, Y: bottom/top)
};

struct Scene {
    Settings s{};
    std::vector<Domain> doms;       // scene order (reference domain_list order)
    std::vector<Receiver> receivers;
    std::vector<Speaker> speakers;
    std::vector<StripRun> runs;     // for every non-rigid domain and updated axis
    bool spectral = false;          // receivers interpolate spectrally (PSTD_RECEIVERS_SPECTRAL)

    void build(const pstd_config* cfg);
    std::vector<StripRun> runs_of(int k, Axis a) const;   // runs of any domain and axis
    int window_for(int n) const;            // window after halving for a strip of n cells
    static int next_pow2(int n);
};

// Reflection / transmission of the low (1) and high (2) interface bands of a
// strip of a domain of density rs between neighbours of density r1 and r2
// (kernel/core/kernel_functions.cpp:37-64, float as the reference);
// pressure strips (vel = false) or velocity strips.
inline void band_coefficients(float rs, float r1, float r2, bool vel, float& R1, float& T1, float& R2, float& T2) {
    float zn1 = r1 / rs, izn1 = rs / r1, zn2 = r2 / rs, izn2 = rs / r2;
    float rlw1 = (zn1 - 1) / (zn1 + 1), tlw1 = (2 * zn1) / (zn1 + 1), tlw2 = (2 * izn1) / (izn1 + 1);
    float rrw1 = (zn2 - 1) / (zn2 + 1), trw1 = (2 * zn2) / (zn2 + 1), trw2 = (2 * izn2) / (izn2 + 1);
    if (vel) { R1 = -rlw1; T1 = tlw1; R2 = -rrw1; T2 = trw1; }
    else     { R1 = rlw1;  T1 = tlw2; R2 = rrw1;  T2 = trw2; }
}

// attenuation profile (FP64 build) of length P (pressure) or P+1 (velocity)
void pml_profile(const Settings& s, bool velocity, bool ascending, std::vector<double>& out);

}  // namespace pstd
