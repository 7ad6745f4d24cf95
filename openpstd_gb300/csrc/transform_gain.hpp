// transform_gain.hpp -- the round-trip gain of the stage kernel's FFT per
// frequency bin, from the rounding of its constants, and the butterfly
// constants themselves (one definition for the device code and this model).
//
// The transform's constants are float: the internal butterfly rotations
// (cos / sin of multiples of pi/16, sqrt(1/2)) and the per-pass twiddle
// tables (or, with computed twiddles, products of a few stored powers).
// cos(pi/8), sin(pi/8) and sqrt(1/2) all round down in float, so every mode
// that passes through them loses a little amplitude, in the forward and the
// inverse transform alike: the forward + inverse round trip of a mode gains
// 1 + g(k) with g about -5e-8 .. -1.2e-7 on average over the bins, nearly the
// same sign for all of them.  Applied in every derivative of every RK stage,
// such a gain scales the discrete wave speed, and the phase error it causes
// grows linearly with the step count (the solve's receiver error against FP64
// would grow 2-3.6x faster than the reference's own float build does).  The
// derivative filter is divided by this gain, bin by bin, when it is built, so
// the device pays nothing.
//
// The gain is taken to first order in the constants' rounding errors, with
// exact arithmetic: a mode of frequency k enters pass p (block M, radix R)
// as a pure pattern of digit d = k_p mod R; the radix-R butterfly maps it to
// its output d with gain dft_gain(R, d); the twiddles of column d multiply
// it by (1 + delta(n1, d)), whose projection on the mode is the mean over n1;
// the inverse passes repeat this with conjugate twiddles.  The model matches
// an exact emulation of the passes (all bins, constants as on the device) to
// 1e-14 for the plans checked; the device's own float arithmetic adds random
// rounding on top, which no table can remove.
#pragma once
#include <cmath>
#include <complex>
#include <vector>

// cos / sin of multiples of pi/8 and pi/16 (radix 8, 16 and 32 butterflies)
#define PSTD_C8 0.92387953251128674f
#define PSTD_S8 0.38268343236508978f
#define PSTD_R2 0.70710678118654752f
#define PSTD_C16 0.98078528040323044913f   // cos(pi/16)
#define PSTD_S16 0.19509032201612826785f   // sin(pi/16)
#define PSTD_C316 0.83146961230254523708f  // cos(3 pi/16)
#define PSTD_S316 0.55557023301960222474f  // sin(3 pi/16)

namespace pstd {
namespace tgain {

using cd = std::complex<double>;

// a * exp(-/+ 2 pi i K / 32) with the device's float constants (tw16 for even K)
inline cd rot32(int K, bool inv, cd a) {
    const double sg = inv ? 1.0 : -1.0;
    if (K == 0) return a;
    if (K == 8) return inv ? cd(-a.imag(), a.real()) : cd(a.imag(), -a.real());
    double c, s;
    if (K % 2 == 0) {
        const int k = K / 2;   // tw16<k>
        const double R2 = PSTD_R2, C8 = PSTD_C8, S8 = PSTD_S8;
        switch (k) {
            case 2: c = R2; s = R2; break;
            case 6: c = -R2; s = R2; break;
            case 1: c = C8; s = S8; break;
            case 3: c = S8; s = C8; break;
            case 5: c = -S8; s = C8; break;
            default: c = -C8; s = S8; break;   // 7
        }
    } else {
        const double C16 = PSTD_C16, S16 = PSTD_S16, C316 = PSTD_C316, S316 = PSTD_S316;
        switch (K) {
            case 1: c = C16; s = S16; break;
            case 3: c = C316; s = S316; break;
            case 5: c = S316; s = C316; break;
            case 7: c = S16; s = C16; break;
            case 9: c = -S16; s = C16; break;
            case 11: c = -S316; s = C316; break;
            case 13: c = -C316; s = S316; break;
            default: c = -C16; s = S16; break;   // 15
        }
    }
    return a * cd(c, sg * s);
}

// the device's recursive radix-R DFT (stage_kernel.cuh: DFT<R>), in place
inline void dft(cd* x, int R, bool inv) {
    if (R == 1) return;
    if (R == 2) {
        const cd a = x[0], b = x[1];
        x[0] = a + b;
        x[1] = a - b;
        return;
    }
    if (R == 4) {
        const cd a = x[0] + x[2], b = x[0] - x[2], c = x[1] + x[3];
        const cd t = x[1] - x[3];
        const cd d = inv ? cd(-t.imag(), t.real()) : cd(t.imag(), -t.real());
        x[0] = a + c;
        x[2] = a - c;
        x[1] = b + d;
        x[3] = b - d;
        return;
    }
    std::vector<cd> e(R / 2), o(R / 2);
    for (int k = 0; k < R / 2; k++) {
        e[k] = x[2 * k];
        o[k] = x[2 * k + 1];
    }
    dft(e.data(), R / 2, inv);
    dft(o.data(), R / 2, inv);
    const int step = 32 / R;   // o[k] * exp(-/+ 2 pi i k / R) = rot32(k * step)
    for (int k = 1; k < R / 2; k++) o[k] = rot32(k * step, inv, o[k]);
    for (int k = 0; k < R / 2; k++) {
        x[k] = e[k] + o[k];
        x[k + R / 2] = e[k] - o[k];
    }
}

// forward gain of output d for the input pattern of digit d, times the
// inverse gain of the impulse at input d projected on that pattern
inline cd dft_round_trip(int R, int d) {
    std::vector<cd> x(R), y(R, cd(0, 0));
    for (int q = 0; q < R; q++) x[q] = std::polar(1.0, 2.0 * M_PI * d * q / R);
    dft(x.data(), R, false);
    const cd gf = x[d] / (double)R;
    y[d] = 1.0;
    dft(y.data(), R, true);
    cd gi = 0;
    for (int q = 0; q < R; q++) gi += y[q] * std::polar(1.0, -2.0 * M_PI * d * q / R);
    return gf * gi / (double)R;
}

inline cd f32(double re, double im) { return cd((double)(float)re, (double)(float)im); }
inline cd tw(double n, int M) { return f32(std::cos(-2.0 * M_PI * n / M), std::sin(-2.0 * M_PI * n / M)); }

// the device's float complex product a * b (cmul): each component one
// rounded product and one fused multiply-add
inline cd mul32(cd a, cd b) {
    const double p = (double)(float)(a.imag() * b.imag()), q = (double)(float)(a.imag() * b.real());
    return cd((double)(float)(a.real() * b.real() - p), (double)(float)(a.real() * b.imag() + q));
}

// twiddle w[n1][k] of a pass (block M, radix R) as the device forms it
// (table entry; computed twiddles: float products of the stored powers,
// stage_kernel.cuh: make_twiddles)
inline cd twiddle(int M, int R, int n1, int k, bool ctw) {
    if (!ctw || R == 2) return tw((double)n1 * k, M);
    const cd w1 = tw(n1, M);
    if (R == 4) {
        const cd wb = tw(2.0 * n1, M);
        const cd v[4] = {1.0, w1, wb, mul32(wb, w1)};
        return v[k];
    }
    if (R == 8) {
        const cd wb = tw(4.0 * n1, M), w2 = mul32(w1, w1), w3 = mul32(w2, w1);
        const cd v[8] = {1.0, w1, w2, w3, wb, mul32(wb, w1), mul32(wb, w2), mul32(wb, w3)};
        return v[k];
    }
    const cd w2 = tw(2.0 * n1, M), w4 = tw(4.0 * n1, M), w8 = tw(8.0 * n1, M);
    const cd w3 = mul32(w2, w1), w12 = mul32(w8, w4);
    const cd lo[4] = {1.0, w1, w2, w3}, hi[4] = {1.0, w4, w8, w12};
    return (k & 3) ? ((k >> 2) ? mul32(hi[k >> 2], lo[k & 3]) : lo[k & 3]) : hi[k >> 2];
}

// Round-trip gain per bin k < L (natural frequency order) of the transform
// with passes radices[0..np): all but the last with twiddle tables, the last
// in registers (lane_pair: split as radix 2 with a float table, then R/2).
inline std::vector<cd> round_trip_gain(int L, const int* radices, int np, bool ctw, bool lane_pair) {
    std::vector<int> rad, kind;   // kind 0: table twiddles; 1: lane-pair table (non-computed)
    for (int p = 0; p < np; p++) {
        if (p == np - 1 && lane_pair) {
            rad.push_back(2);
            kind.push_back(1);
            rad.push_back(radices[p] / 2);
        } else {
            rad.push_back(radices[p]);
            kind.push_back(0);
        }
    }
    std::vector<cd> g(L, cd(1, 0));
    std::vector<int> kk(L);
    for (int k = 0; k < L; k++) kk[k] = k;
    int M = L;
    for (size_t p = 0; p < rad.size(); p++) {
        const int R = rad[p];
        std::vector<cd> dg(R), col(R, cd(0, 0));
        for (int d = 0; d < R; d++) dg[d] = dft_round_trip(R, d);
        const bool twiddled = p + 1 < rad.size();
        if (twiddled) {
            const int Q = M / R;
            for (int d = 0; d < R; d++) {
                cd s = 0;
                for (int n1 = 0; n1 < Q; n1++) {
                    const cd w = twiddle(M, R, n1, d, ctw && kind[p] == 0);
                    s += w / std::polar(1.0, -2.0 * M_PI * n1 * d / M);
                }
                col[d] = s / (double)Q;
            }
        }
        for (int k = 0; k < L; k++) {
            const int d = kk[k] % R;
            g[k] *= dg[d];
            if (twiddled) g[k] *= col[d] * std::conj(col[d]);
            kk[k] = (kk[k] - d) / R;
        }
        if (twiddled) M /= R;
    }
    return g;
}

}  // namespace tgain
}  // namespace pstd
