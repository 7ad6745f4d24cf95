// spectral_receivers.hpp -- host plan of the spectral receivers.
//
// A spectral receiver at grid location (gx, gy), in the cell (ix, iy) of its
// container D, samples p0 at the point itself (the interpolation the
// reference's Receiver::compute_with_si, kernel/core/Receiver.cpp:85-121, was
// meant to do; it is disabled there, :48, and shifts by the integer grid
// location, :41).  Both passes use the windowed strip transform of the
// pressure derivative (Domain::calc, kernel/core/Domain.cpp:95-391;
// spatderp3, kernel/core/kernel_functions.cpp:123-318) with the factors
// exp(i k delta dx) (the shift by delta cells) in place of the derivative's:
//
//   x pass: the rows of D and the W_y rows of D's low / high y neighbours
//           nearest to D are shifted along x by gx - ix, each in its own
//           domain's x strips (its own x neighbours, bands and window), and
//           sampled at column ix;
//   y pass: the column formed by those samples is shifted along y by gy - iy
//           in D's y strip through column ix and sampled at row iy.
//
// Both passes are linear in p0, and for a fixed receiver the maps are fixed:
// out[m] = sum_j buf[j] g[(W + m - j) mod L], buf the windowed strip (band of
// the low neighbour, blended with the strip's reversed start; the strip; the
// high band, blended with the reversed end; zeros), g the real inverse
// transform of the shift factors (c2r ignoring the Nyquist imaginary part):
//   g[t] = (1 + 2 sum_{k=1}^{L/2-1} cos(2 pi k (t + delta) / L) + cos(pi delta) (-1)^t) / L.
// The plan folds bands, reflection / transmission and window into one weight
// per cell (double, rounded to float once); the device evaluates every row as
// a dot product (si_rows_kernel) and sums the weighted rows per receiver.
#pragma once

#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <vector>

#include "device.cuh"
#include "scene.hpp"

namespace pstd {

// g[t], t < L, of the shift by delta cells (closed form of the cosine sum)
inline std::vector<double> shift_kernel(int L, double delta) {
    const int M = L / 2;
    std::vector<double> g(L);
    for (int t = 0; t < L; t++) {
        const double th = 2.0 * M_PI * (t + delta) / L;
        const double h = std::sin(0.5 * th);
        const double s = std::fabs(h) < 1e-12 ? (double)(M - 1) : std::sin((M - 0.5) * th) / (2.0 * h) - 0.5;
        g[t] = (1.0 + 2.0 * s + std::cos(M_PI * delta) * ((t & 1) ? -1.0 : 1.0)) / L;
    }
    return g;
}

// Weights of output m of the shifted pressure strip of domain `k` along axis a
// over [low band W | strip n | high band W] (low band: the neighbour's last W
// cells; high band: its first W), for the run r (neighbours d1, d2).
// win: the 2W+1 window coefficients.
inline std::vector<double> shifted_strip_weights(const Scene& sc, int k, Axis a, const StripRun& r, int m, double delta,
                                                 const float* win) {
    const Domain& d = sc.doms[k];
    const int n = d.len(a), W = sc.window_for(n), L = Scene::next_pow2(n + 2 * W);
    const std::vector<double> g = shift_kernel(L, delta);
    auto G = [&](int t) { t %= L; return g[t < 0 ? t + L : t]; };
    float R1, T1, R2, T2;
    band_coefficients(d.rho, r.d1 >= 0 ? sc.doms[r.d1].rho : d.rho, r.d2 >= 0 ? sc.doms[r.d2].rho : d.rho, false, R1,
                      T1, R2, T2);
    std::vector<double> w(2 * W + n, 0.0);
    for (int i = 0; i < n; i++) w[W + i] = G(m - i);
    for (int j = 0; j < W; j++) {
        const double lo = (double)win[j] * G(W + m - j);          // buf[j]
        const double hi = (double)win[W + 1 + j] * G(m - n - j);  // buf[W + n + j]
        if (r.d1 >= 0) w[j] += T1 * lo;
        w[W + W - 1 - j] += R1 * lo;
        if (r.d2 >= 0) w[W + n + j] += T2 * hi;
        w[W + n - 1 - j] += R2 * hi;
    }
    return w;
}

inline const StripRun& run_holding(const std::vector<StripRun>& runs, int strip) {
    for (const StripRun& r : runs)
        if (r.first <= strip && strip < r.first + r.count) return r;
    throw SceneError(PSTD_ERR_UNSUPPORTED, "spectral receiver: a strip without an interface combination");
}

struct SpectralPlan {
    std::vector<DevSiRow> rows;
    std::vector<float> weights;
    std::vector<int> first;   // first row of every receiver (+ the end, once complete)
};

// Append the stencil rows of every receiver of scene `sc` (domain indices
// offset by `base`); window(W) returns the 2W+1 coefficients of window W.
inline void plan_spectral_receivers(const Scene& sc, int base, const std::function<const float*(int)>& window,
                                    SpectralPlan& plan) {
    for (const Receiver& q : sc.receivers) {
        plan.first.push_back((int)plan.rows.size());
        const int D = q.dom;
        const Domain& dd = sc.doms[D];
        const int ix = (int)q.gx, iy = (int)q.gy;
        const double fx = (double)q.gx - ix, fy = (double)q.gy - iy;
        const int mx = ix - dd.x0, my = iy - dd.y0;
        // y pass: D's y strip through column mx
        const std::vector<StripRun> yruns = sc.runs_of(D, AX_Y);
        const StripRun& yr = run_holding(yruns, mx);
        const int Wy = sc.window_for(dd.ny);
        const std::vector<double> yw = shifted_strip_weights(sc, D, AX_Y, yr, my, fy, window(Wy));
        // the stencil rows: (domain, row, y weight)
        struct Row { int dom, row; double w; };
        std::vector<Row> rs;
        if (yr.d1 >= 0)
            for (int j = 0; j < Wy; j++) rs.push_back({yr.d1, sc.doms[yr.d1].ny - Wy + j, yw[j]});
        for (int i = 0; i < dd.ny; i++) rs.push_back({D, i, yw[Wy + i]});
        if (yr.d2 >= 0)
            for (int j = 0; j < Wy; j++) rs.push_back({yr.d2, j, yw[Wy + dd.ny + j]});
        // x pass: one weight vector per (domain, x run) the rows use
        std::map<std::pair<int, int>, int> woff;
        std::map<int, std::vector<StripRun>> xruns;
        for (const Row& r : rs) {
            const Domain& e = sc.doms[r.dom];
            auto it = xruns.find(r.dom);
            if (it == xruns.end()) it = xruns.emplace(r.dom, sc.runs_of(r.dom, AX_X)).first;
            const StripRun& xr = run_holding(it->second, r.row);
            const int ri = (int)(&xr - it->second.data());
            const int Wx = sc.window_for(e.nx), cx = ix - e.x0;
            if (cx < 0 || cx >= e.nx)
                throw SceneError(PSTD_ERR_UNSUPPORTED, "spectral receiver: column outside a y neighbour");
            auto key = std::make_pair(r.dom, ri);
            auto wi = woff.find(key);
            if (wi == woff.end()) {
                const std::vector<double> w = shifted_strip_weights(sc, r.dom, AX_X, xr, cx, fx, window(Wx));
                wi = woff.emplace(key, (int)plan.weights.size()).first;
                for (double v : w) plan.weights.push_back((float)v);
            }
            DevSiRow s;
            std::memset(&s, 0, sizeof s);
            s.dom = base + r.dom;
            s.row = r.row;
            s.d1 = xr.d1 >= 0 ? base + xr.d1 : -1;
            s.d2 = xr.d2 >= 0 ? base + xr.d2 : -1;
            s.r1 = xr.d1 >= 0 ? e.y0 + r.row - sc.doms[xr.d1].y0 : 0;
            s.r2 = xr.d2 >= 0 ? e.y0 + r.row - sc.doms[xr.d2].y0 : 0;
            s.W = Wx;
            s.w = wi->second;
            s.yw = (float)r.w;
            plan.rows.push_back(s);
        }
    }
}

}  // namespace pstd
