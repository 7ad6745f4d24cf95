// device.cuh -- data layout shared by the host plan and the sm_103a kernels.
//
// Field storage.  Three rotating state sets (A, B, C) of identical layout hold
// px, py, vx, vy of every non-rigid domain; rows are padded to a multiple of
// 32 floats (128 B):
//   px, py : Ny rows x Nx      (pitch_p)
//   vx     : Ny rows x (Nx+1)  (pitch_vx)
//   vy     : (Ny+1) rows x Nx  (pitch_vy)
// A time step reads the stage-start set P and writes the six RK stages
// alternately into the two other sets; the last stage's set becomes P of the
// next step, so there is no push_values copy (kernel/Solver.cpp:73-76).
//
// p0 is not stored per stage: every stage forms p0 = px + py of the previous
// stage while loading (kernel/Solver.cpp:114-116 computes exactly that sum).
// One p0 array per domain holds the values the reference reads at the first
// stage of a step where they differ from px + py: the speaker initial p0 at
// the very first step (kernel/core/Speaker.cpp:35) and, for PML domains, p0
// from before the PML multiply (kernel/Solver.cpp:85 leaves p0 stale).
//
// Rigid domains are never RK-updated (kernel/Solver.cpp:101,110): their
// fields live once in a fixed buffer that only the per-step PML kernel
// touches.
#pragma once
#include <cstdint>

namespace pstd {

struct DevDomain {
    int nx, ny;
    int pitch_p, pitch_vx, pitch_vy;
    int att_xp, att_xv, att_yp, att_yv;   // offsets into the attenuation table, -1 = none
    int pml;                              // PML domain (stale p0 at the first stage of a step)
    int fixed;                            // rigid: fields in the fixed buffer
    int scene;                            // scene of a batch (index of its first-step flag)
    long long o_px, o_py, o_vx, o_vy;     // float offsets inside a state set (or the fixed buffer)
    long long o_p0;                       // float offset in the p0 array
    float rho;                            // domain density (float, as the reference)
    float c2;                             // c1*c1 (float)
    float cdt[6];                         // dt * rk_coefficient[k] (float)
};

enum JobKind : int {
    JK_VEL = 1,    // derivative of the velocity strip (updates px / py); else of p0 (updates vx / vy)
    JK_Y = 2,      // y-direction strips (columns); else x-direction (rows)
    JK_COPY = 4,   // axis not updated (should_update == false): carry the axis' fields through
};

// Up to 2*CS adjacent strips of one domain that share both interface
// neighbours; one CTA per job.
struct DevJob {
    int dom, first, count, kind;
    int W;            // window length (after halving)
    int d1, d2;       // neighbour supplying the low / high band, -1 = none (zero band)
    int o1, o2;       // index of strip `first` inside d1 / d2
    float R1, T1, R2, T2;   // reflection / transmission of the two bands
    int dtab;         // float2 offset of the permuted derivative filter
    int wtab;         // float offset of the 2W+1 window coefficients
    int L;            // transform length (0 for a copy job)
    int ttab;         // float2 offset of the twiddle tables of the job's radix plan
};

struct DevReceiver {
    int dom, row, col;
};

// One row of a spectral receiver's stencil: the row's p0 shifted along x to
// the receiver's column (a weighted sum over the row and the bands of its x
// neighbours), times the row's weight in the y shift.
struct DevSiRow {
    int dom, row;     // the row (y index inside dom)
    int d1, d2;       // x neighbours supplying the bands, -1 = none
    int r1, r2;       // the same row inside d1 / d2
    int W;            // band width
    int w;            // weights: W (d1 cells nx1-W..nx1-1), nx (the row), W (d2 cells 0..W-1)
    float yw;         // weight of the row in the y shift
};

struct DevSpeaker {
    float x, y;
};

// Receiver of a scene in the serving loop: its samples go to the scene's own
// ring (step-major, `stride` receivers per step) at the scene's own step count.
struct DevSrvReceiver {
    int dom, row, col, slot;
    long long ring;   // float offset of the scene's ring in the auxiliary arena
    int stride, index;
};

}  // namespace pstd
