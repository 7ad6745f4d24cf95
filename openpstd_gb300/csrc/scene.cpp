// scene.cpp -- host-side scene construction (see scene.hpp).
//
// Follows the reference's scene rules step by step so that the device solve
// sees the same domains, neighbours and flags as openPSTD's CPU PSTDKernel:
//   world->grid scaling and T/B edge swap    kernel/PSTDKernel.cpp:73-98,170-190
//   neighbour detection                      kernel/core/Scene.cpp:297-380
//   automatic PML + corner PML + merging     kernel/core/Scene.cpp:41-251
//   vacant edge runs                         kernel/core/Domain.cpp:543-584
//   update directions                        kernel/core/Domain.cpp:587-616
//   PML orientation flags                    kernel/core/Domain.cpp:644-714
//   speakers / receivers                     kernel/core/Scene.cpp:254-279, kernel/core/Receiver.cpp:34-83
//   interface combination per strip          kernel/core/Domain.cpp:147-189
// Layouts on which the reference reads undefined memory are rejected with
// PSTD_ERR_UNSUPPORTED and a message naming the cause.
#include "scene.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <map>
#include <tuple>

namespace pstd {

static const float kEps = 1e-5f;   // kernel/core/kernel_functions.h:65

float Settings::dt() const { return tfactRK * dx / c1; }

int Settings::window() const {
    int t = (int)std::round((patcherror * 0.7 - 17) / 2.);
    return (int)std::round(t * 2);
}

int Settings::framecount() const { return (int)(calctime / dt()); }

int Scene::next_pow2(int n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

int Scene::window_for(int n) const {
    int w = s.window();
    while (w > n) w /= 2;
    return w;
}

namespace {

Side opposite(Side s) {
    switch (s) {
        case S_LEFT: return S_RIGHT;
        case S_RIGHT: return S_LEFT;
        case S_TOP: return S_BOTTOM;
        default: return S_TOP;
    }
}
Axis axis_of(Side s) { return (s == S_LEFT || s == S_RIGHT) ? AX_X : AX_Y; }

struct Builder {
    Settings s;
    std::vector<Domain> pool;     // every domain ever created, stable indices
    std::vector<int> order;       // scene order (pool indices)
    int next_id = 0;

    bool contains(const std::vector<int>& v, int x) const { return std::find(v.begin(), v.end(), x) != v.end(); }

    bool listed_neighbour(int a, int b) const {
        for (int k = 0; k < 4; k++) if (contains(pool[a].nb[k], b)) return true;
        return false;
    }

    int create(float alpha, int x0, int y0, int nx, int ny, int parent) {
        Domain d;
        d.id = next_id++;
        d.alpha = alpha;
        d.x0 = x0; d.y0 = y0; d.nx = nx; d.ny = ny;
        float r = std::sqrt(1.0f - alpha);
        d.impedance = -((r + 1) / (r - 1));
        d.rigid = d.impedance > 1000;
        d.rho = d.rigid ? 1e30f : s.rho * d.impedance;
        if (parent >= 0) {
            d.pml = true;
            d.parents.push_back(parent);
            d.secondary = pool[parent].pml;
        }
        pool.push_back(d);
        return (int)pool.size() - 1;
    }

    // overlap length of the strip ranges of two domains along axis a
    static int overlap(const Domain& p, const Domain& q, Axis a) {
        int lo = std::max(p.lo(a), q.lo(a)), hi = std::min(p.hi(a), q.hi(a));
        return std::max(0, hi - lo);
    }

    void add(int ni) {
        for (int ei : order) {
            Domain& n = pool[ni];
            Domain& e = pool[ei];
            if (n.secondary && e.secondary) continue;
            if ((n.secondary && !e.pml) || (e.secondary && !n.pml)) continue;
            if (n.pml && e.pml) {
                bool serves_new = contains(e.parents, ni), new_serves = contains(n.parents, ei);
                bool direct = (n.secondary && new_serves) || (e.secondary && serves_new);
                if (!direct) {
                    if (e.parents.size() != 1 || n.parents.size() != 1) continue;
                    if (!listed_neighbour(e.parents[0], n.parents[0])) continue;
                    if (!listed_neighbour(n.parents[0], e.parents[0])) continue;
                }
            }
            int side = -1;
            if (n.x1() == e.x0) side = S_RIGHT;
            else if (n.x0 == e.x1()) side = S_LEFT;
            else if (n.y1() == e.y0) side = S_BOTTOM;
            else if (n.y0 == e.y1()) side = S_TOP;
            if (side < 0) continue;
            bool e_foreign = e.pml && !n.pml && !contains(e.parents, ni);
            bool n_foreign = n.pml && !e.pml && !contains(n.parents, ei);
            if (e_foreign || n_foreign) continue;
            if (overlap(n, e, axis_of((Side)side)) == 0) continue;
            pool[ni].nb[side].push_back(ei);
            pool[ei].nb[opposite((Side)side)].push_back(ni);
        }
        order.push_back(ni);
    }

    // the part of an edge not covered by neighbours, as one run [lo, hi) (or none)
    bool vacant_run(int di, Side side, int& lo, int& hi) {
        const Domain& d = pool[di];
        Axis a = axis_of(side);
        int a0 = d.lo(a), a1 = d.hi(a);
        std::vector<char> free_(a1 - a0, 1);
        for (int o : d.nb[side]) {
            const Domain& q = pool[o];
            for (int v = std::max(a0, q.lo(a)); v < std::min(a1, q.hi(a)); v++) free_[v - a0] = 0;
        }
        int runs = 0;
        lo = hi = 0;
        for (int v = 0; v < a1 - a0; v++) {
            if (free_[v] && (v == 0 || !free_[v - 1])) { runs++; lo = a0 + v; }
            if (free_[v]) hi = a0 + v + 1;
        }
        if (runs > 1)
            throw SceneError(PSTD_ERR_UNSUPPORTED,
                             "domain " + std::to_string(d.id) + " has an edge with more than one uncovered run; "
                             "the reference's vacant-range table leaves rows uninitialised for that layout");
        return runs == 1;
    }

    void add_pml() {
        const int P = s.pml_cells;
        const Side seq[4] = {S_LEFT, S_TOP, S_RIGHT, S_BOTTOM};
        std::vector<int> primaries;
        std::vector<std::pair<int, Side>> corners;
        std::vector<int> air = order;
        for (int ai : air) {
            if (pool[ai].pml) continue;
            for (int i = 0; i < 4; i++) {
                Side side = seq[i];
                int lo, hi;
                if (!vacant_run(ai, side, lo, hi)) continue;
                const Domain a = pool[ai];
                float alpha = a.edge_alpha[side];
                float palpha = std::max(alpha, kEps);
                int x0, y0, nx, ny;
                switch (side) {
                    case S_LEFT: x0 = a.x0 - P; y0 = lo; nx = P; ny = hi - lo; break;
                    case S_RIGHT: x0 = a.x1(); y0 = lo; nx = P; ny = hi - lo; break;
                    case S_TOP: x0 = lo; y0 = a.y0 - P; nx = hi - lo; ny = P; break;
                    default: x0 = lo; y0 = a.y1(); nx = hi - lo; ny = P; break;
                }
                bool full = lo == a.lo(axis_of(side)) && hi == a.hi(axis_of(side));
                int pi = create(palpha, x0, y0, nx, ny, ai);
                pool[pi].local = !full;
                primaries.push_back(pi);
                if (alpha > 0 && full) {
                    for (int k : {(i + 1) % 4, (i + 3) % 4}) {
                        Side second = seq[k];
                        float oa = a.edge_alpha[second];
                        float calpha = std::min(std::max(kEps, oa), std::max(kEps, palpha));
                        const Domain& p = pool[pi];
                        int cx = p.x0, cy = p.y0;
                        if (second == S_LEFT) cx -= P;
                        else if (second == S_RIGHT) cx += p.nx;
                        else if (second == S_TOP) cy -= P;
                        else cy += p.ny;
                        int ci = create(calpha, cx, cy, P, P, pi);
                        corners.push_back({ci, second});
                    }
                }
            }
        }
        for (int pi : primaries) add(pi);
        // group surviving corner candidates by their rectangle (ordered by x0, y0, x1, y1)
        std::map<std::tuple<int, int, int, int>, std::vector<int>> groups;
        for (auto& c : corners) {
            const Domain& cd = pool[c.first];
            if (!pool[cd.parents[0]].nb[c.second].empty()) continue;
            groups[std::make_tuple(cd.x0, cd.y0, cd.x1(), cd.y1())].push_back(c.first);
        }
        auto grandparent = [&](int ci) -> int {
            int p = (pool[ci].pml && pool[ci].parents.size() == 1) ? pool[ci].parents[0] : -1;
            if (p < 0) return -1;
            return (pool[p].pml && pool[p].parents.size() == 1) ? pool[p].parents[0] : -1;
        };
        std::vector<int> final_corners;
        for (auto& g : groups) {
            auto& v = g.second;
            if (v.size() == 1) { final_corners.push_back(v[0]); continue; }
            std::vector<int> merged;
            for (size_t i = 0; i < v.size(); i++) {
                for (size_t j = i + 1; j < v.size(); j++) {
                    if (contains(merged, v[i]) || contains(merged, v[j])) continue;
                    int gi = grandparent(v[i]), gj = grandparent(v[j]);
                    if (gi >= 0 && gj >= 0 && pool[gi].id == pool[gj].id) {
                        merged.push_back(v[i]);
                        merged.push_back(v[j]);
                        for (int q : pool[v[j]].parents) pool[v[i]].parents.push_back(q);
                        final_corners.push_back(v[i]);
                    }
                }
            }
            for (int c : v) if (!contains(merged, c)) final_corners.push_back(c);
        }
        for (int c : final_corners) add(c);
    }

    void update_flags(int di) {
        Domain& d = pool[di];
        int total = 0, pmls = 0;
        for (int k = 0; k < 4; k++)
            for (int o : d.nb[k]) { total++; if (pool[o].pml) pmls++; }
        for (int ax = 0; ax < 2; ax++) {
            bool up = true;
            if (total - pmls == 1 && d.pml) {
                // has_horizontal_attenuation is read before it is assigned in the
                // reference; it is taken as false (value-initialised).
                const bool hha = false;
                if (hha && ax == AX_X) up = true;
                else if (!hha && ax == AX_Y) up = true;
                else if (d.local) up = false;
                else {
                    for (int k = 0; k < 4; k++) {
                        if (d.nb[k].size() == 1 && !pool[d.nb[k][0]].pml)
                            up = !pool[d.nb[k][0]].edge_lr[k];
                    }
                }
            }
            d.update[ax] = up;
        }
    }

    void attenuation_flags(int di) {
        Domain& d = pool[di];
        int total = 0;
        for (int k = 0; k < 4; k++) total += (int)d.nb[k].size();
        auto pml_count = [&](Side sd) {
            int n = 0;
            for (int o : d.nb[sd]) if (pool[o].pml) n++;
            return n;
        };
        bool corner = false, hha, rev0, rev1 = false;
        if (d.secondary) {
            corner = total == 2;
            hha = !d.nb[S_LEFT].empty() || !d.nb[S_RIGHT].empty();
            if (corner) {
                if (!(hha && (!d.nb[S_TOP].empty() || !d.nb[S_BOTTOM].empty())))
                    throw SceneError(PSTD_ERR_UNSUPPORTED, "corner PML without a horizontal and a vertical neighbour");
                rev0 = !d.nb[S_LEFT].empty();
                rev1 = !d.nb[S_BOTTOM].empty();
            } else {
                rev0 = !d.nb[S_LEFT].empty() || !d.nb[S_BOTTOM].empty();
            }
        } else {
            bool air_l = !d.nb[S_LEFT].empty() && pml_count(S_LEFT) == 0;
            bool air_r = !d.nb[S_RIGHT].empty() && pml_count(S_RIGHT) == 0;
            bool air_b = !d.nb[S_BOTTOM].empty() && pml_count(S_BOTTOM) == 0;
            hha = air_l || air_r;
            rev0 = air_l || air_b;
        }
        if (corner) {
            d.att_x = true; d.asc_x = rev0;
            d.att_y = true; d.asc_y = rev1;
        } else if (hha) {
            d.att_x = true; d.asc_x = rev0;
        } else {
            d.att_y = true; d.asc_y = rev0;
        }
        if (d.att_x && d.nx != s.pml_cells)
            throw SceneError(PSTD_ERR_UNSUPPORTED, "x attenuation profile does not fit PML domain " + std::to_string(d.id));
        if (d.att_y && d.ny != s.pml_cells)
            throw SceneError(PSTD_ERR_UNSUPPORTED, "y attenuation profile does not fit PML domain " + std::to_string(d.id));
    }
};

}  // namespace

void pml_profile(const Settings& s, bool velocity, bool ascending, std::vector<double>& out) {
    // kernel/core/Domain.cpp:743-768, built in double precision
    const int P = s.pml_cells;
    const double dt = (double)s.dt();
    int n = velocity ? P + 1 : P;
    out.resize(n);
    for (int i = 0; i < n; i++) {
        double r = velocity ? (double)i / P : (i + 0.5) / P;
        double r4 = r * r * r * r;
        out[i] = velocity ? std::exp(-(double)s.rho * (double)s.ampMax * r4 * dt)
                          : std::exp(-(double)s.ampMax * r4 * dt / (double)s.rho);
    }
    if (!ascending) std::reverse(out.begin(), out.end());
}

void Scene::build(const pstd_config* cfg) {
    if (!cfg) throw SceneError(PSTD_ERR_INVALID, "null configuration");
    const pstd_settings& st = cfg->settings;
    s.calctime = st.calctime; s.c1 = st.c1; s.ampMax = st.ampMax; s.rho = st.rho;
    s.patcherror = st.patcherror; s.tfactRK = st.tfactRK; s.dx = st.gridSpacing;
    s.band_width = st.band_width; s.pml_cells = st.PMLCells; s.save_nth = st.SaveNth;
    if (st.n_rk_coefficients != 6) throw SceneError(PSTD_ERR_INVALID, "the RK update needs exactly 6 coefficients");
    for (int i = 0; i < 6; i++) s.rk[i] = st.rk_coefficients[i];
    if (!(s.dx > 0) || !(s.c1 > 0) || !(s.tfactRK > 0) || !(s.rho > 0))
        throw SceneError(PSTD_ERR_INVALID, "grid spacing, sound speed, CFL factor and density must be positive");
    if (s.save_nth <= 0) throw SceneError(PSTD_ERR_INVALID, "SaveNth must be positive");
    spectral = st.spectral_interpolation == PSTD_RECEIVERS_SPECTRAL;
    if (s.window() <= 0) throw SceneError(PSTD_ERR_INVALID, "patch error gives an empty window");
    if (cfg->n_domains <= 0 || !cfg->domains) throw SceneError(PSTD_ERR_INVALID, "no domains");
    if (s.pml_cells <= 0) throw SceneError(PSTD_ERR_INVALID, "PMLCells must be positive");

    Builder b;
    b.s = s;
    std::vector<int> air;
    for (int i = 0; i < cfg->n_domains; i++) {
        const pstd_domain_conf& c = cfg->domains[i];
        int x0 = (int)(c.top_left[0] / s.dx), y0 = (int)(c.top_left[1] / s.dx);
        int nx = (int)(c.size[0] / s.dx), ny = (int)(c.size[1] / s.dx);
        if (nx <= 0 || ny <= 0) throw SceneError(PSTD_ERR_INVALID, "domain " + std::to_string(i) + " is empty on the grid");
        int di = b.create(1.f, x0, y0, nx, ny, -1);
        Domain& d = b.pool[di];
        // DomainConf T/B are swapped into the grid's TOP (small y) / BOTTOM
        d.edge_alpha[S_LEFT] = c.L.absorption;  d.edge_lr[S_LEFT] = c.L.lr != 0;
        d.edge_alpha[S_RIGHT] = c.R.absorption; d.edge_lr[S_RIGHT] = c.R.lr != 0;
        d.edge_alpha[S_TOP] = c.B.absorption;   d.edge_lr[S_TOP] = c.B.lr != 0;
        d.edge_alpha[S_BOTTOM] = c.T.absorption; d.edge_lr[S_BOTTOM] = c.T.lr != 0;
        air.push_back(di);
    }
    for (int di : air) b.add(di);
    b.add_pml();
    for (int di : b.order) b.update_flags(di);
    for (int di : b.order) if (b.pool[di].pml) b.attenuation_flags(di);

    // scene order and index remapping
    std::vector<int> to_scene(b.pool.size(), -1);
    for (size_t k = 0; k < b.order.size(); k++) to_scene[b.order[k]] = (int)k;
    doms.clear();
    for (int pi : b.order) {
        Domain d = b.pool[pi];
        for (int k = 0; k < 4; k++) for (int& o : d.nb[k]) o = to_scene[o];
        for (int& o : d.parents) o = (o >= 0 && o < (int)to_scene.size()) ? to_scene[o] : -1;
        doms.push_back(d);
    }

    // speakers (kernel/core/Scene.cpp:267-279): grid coordinate minus half a cell
    speakers.clear();
    for (int i = 0; i < cfg->n_speakers; i++) {
        float gx = cfg->speakers[3 * i] / s.dx, gy = cfg->speakers[3 * i + 1] / s.dx;
        speakers.push_back({gx - 0.5f, gy - 0.5f});
    }
    // receivers (kernel/core/Scene.cpp:254-265): last non-PML domain containing the point
    receivers.clear();
    for (int i = 0; i < cfg->n_receivers; i++) {
        float gx = cfg->receivers[3 * i] / s.dx, gy = cfg->receivers[3 * i + 1] / s.dx;
        int container = -1;
        for (size_t k = 0; k < doms.size(); k++) {
            const Domain& d = doms[k];
            if (d.pml) continue;
            if ((float)d.x0 <= gx && gx <= (float)d.x1() && (float)d.y0 <= gy && gy <= (float)d.y1())
                container = (int)k;
        }
        if (container < 0) throw SceneError(PSTD_ERR_INVALID, "receiver " + std::to_string(i) + " lies outside every domain");
        const Domain& d = doms[container];
        int rx = (int)gx - d.x0, ry = (int)gy - d.y0;
        if (spectral) {
            // the interpolated point (gx, gy) lies in the cell (rx, ry) of the container, at x offset rx
            if (rx < 0 || ry < 0 || rx >= d.nx || ry >= d.ny)
                throw SceneError(PSTD_ERR_UNSUPPORTED,
                                 "receiver " + std::to_string(i) + " lies on the far edge of its domain (no cell to interpolate from)");
        } else if (rx < 0 || ry < 0 || rx >= d.ny || ry >= d.nx) {
            throw SceneError(PSTD_ERR_UNSUPPORTED,
                             "receiver " + std::to_string(i) + " falls outside p0 under the reference's lookup p0(x offset, y offset)");
        }
        receivers.push_back({i, container, rx, ry, gx, gy});
    }

    // strip runs: the interface combination of every row (X) / column (Y)
    runs.clear();
    for (size_t k = 0; k < doms.size(); k++) {
        const Domain& d = doms[k];
        if (d.rigid) continue;
        for (int ax = 0; ax < 2; ax++) {
            if (!d.update[ax]) continue;
            std::vector<StripRun> r = runs_of((int)k, (Axis)ax);
            runs.insert(runs.end(), r.begin(), r.end());
        }
    }
}

// The runs of one domain and axis: Domain::calc's loop over (low, high)
// neighbour pairs (kernel/core/Domain.cpp:95-391), where every pair claims the
// contiguous span [min, max] of the strips it still finds unclaimed.
std::vector<StripRun> Scene::runs_of(int k, Axis a) const {
    std::vector<StripRun> out;
    const Domain& d = doms[k];
    int n = d.len(a);
    int W = window_for(n);
    for (int extra = 0; extra < 2; extra++) {   // pressure (n) and velocity (n+1) strips
        int m = n + extra + 2 * W;
        int L = next_pow2(m);
        int Ld = next_pow2(2 * W + n + (extra ? 0 : 1));
        if (L != Ld)
            throw SceneError(PSTD_ERR_UNSUPPORTED,
                             "domain " + std::to_string(d.id) + ": N+2W is a power of two, so the reference's transform "
                             "length and derivative-factor length disagree");
    }
    const std::vector<int>& lows = (a == AX_X) ? d.nb[S_LEFT] : d.nb[S_BOTTOM];
    const std::vector<int>& highs = (a == AX_X) ? d.nb[S_RIGHT] : d.nb[S_TOP];
    int a0 = d.lo(a), a1 = d.hi(a);
    std::vector<char> remaining(a1 - a0, 1);
    std::vector<std::pair<int, int>> assign(a1 - a0, {INT_MIN, INT_MIN});
    for (size_t i = 0; i <= lows.size(); i++) {
        int d1 = i < lows.size() ? lows[i] : -1;
        for (size_t j = 0; j <= highs.size(); j++) {
            int d2 = j < highs.size() ? highs[j] : -1;
            int lo = a0, hi = a1;
            if (d1 >= 0) { lo = std::max(lo, doms[d1].lo(a)); hi = std::min(hi, doms[d1].hi(a)); }
            if (d2 >= 0) { lo = std::max(lo, doms[d2].lo(a)); hi = std::min(hi, doms[d2].hi(a)); }
            int smin = INT_MAX, smax = INT_MIN;
            for (int v = lo; v < hi; v++) {
                if (!remaining[v - a0]) continue;
                remaining[v - a0] = 0;
                smin = std::min(smin, v);
                smax = std::max(smax, v);
            }
            if (smin > smax) continue;
            for (int nbi : {d1, d2}) {
                if (nbi < 0) continue;
                const Domain& q = doms[nbi];
                if (smin < q.lo(a) || smax + 1 > q.hi(a))
                    throw SceneError(PSTD_ERR_UNSUPPORTED,
                                     "domain " + std::to_string(d.id) + ": an interface span runs past neighbour " +
                                     std::to_string(q.id) + " (the reference reads outside its arrays)");
                if (q.len(a) < W)
                    throw SceneError(PSTD_ERR_UNSUPPORTED,
                                     "neighbour " + std::to_string(q.id) + " is narrower than the window of domain " +
                                     std::to_string(d.id));
            }
            for (int v = smin; v <= smax; v++) assign[v - a0] = {d1, d2};
        }
    }
    int start = 0;
    for (int v = 1; v <= a1 - a0; v++) {
        if (v == a1 - a0 || assign[v] != assign[start]) {
            out.push_back({k, a, start, v - start, assign[start].first, assign[start].second});
            start = v;
        }
    }
    return out;
}

}  // namespace pstd
