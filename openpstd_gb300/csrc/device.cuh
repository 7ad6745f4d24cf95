// device.cuh -- data layout shared by the host plan and the sm_103a kernels.
//
// Field storage: three state sets (A, B, C) of identical layout.  Every domain
// owns five row-major arrays in each set, rows padded to a multiple of 32
// floats (128 B):
//   p0, px, py : Ny rows x Nx      (pitch_p)
//   vx         : Ny rows x (Nx+1)  (pitch_vx)
//   vy         : (Ny+1) rows x Nx  (pitch_vy)
// A time step reads the stage-start set P and writes the six RK stages
// alternately into the two other sets; the last stage's set becomes P of the
// next step, so no push_values copy is made (kernel/Solver.cpp:73-76 copies).
#pragma once
#include <cstdint>

namespace pstd {

struct DevDomain {
    int nx, ny;
    int pitch_p, pitch_vx, pitch_vy;
    int att_xp, att_xv, att_yp, att_yv;   // offsets into the attenuation table, -1 = none
    int pml;
    long long o_p0, o_px, o_py, o_vx, o_vy;   // float offsets inside a state set
    float rho;       // domain density (float, as the reference)
    float c2;        // c1*c1 (float)
    float cdt[6];    // dt * rk_coefficient[k] (float)
};

enum JobKind : int {
    JK_VEL = 1,   // derivative of the velocity strip (updates px / py); else of p0 (updates vx / vy)
    JK_Y = 2,     // y-direction strips (columns); else x-direction (rows)
};

// A batch of at most 2*CS adjacent strips of one domain that share the same
// interface neighbours; one CTA per job.
struct DevJob {
    int dom, first, count, kind;
    int W;            // window length (after halving)
    int d1, d2;       // neighbour supplying the low / high band, -1 = none (zero band)
    int o1, o2;       // index of strip `first` inside d1 / d2
    float R1, T1, R2, T2;   // reflection / transmission of the two bands
    int dtab;         // float2 offset of the permuted derivative filter
    int wtab;         // float offset of the 2W+1 window coefficients
};

// A domain whose fields are only carried through one pass (rigid domain or
// should_update == false along that axis).
struct DevCopy {
    int dom, kind;    // kind: JK_Y or 0
};

struct DevReceiver {
    int dom, row, col;
};

struct DevSpeaker {
    float x, y;
};

}  // namespace pstd
