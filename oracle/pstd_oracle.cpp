// pstd_oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// CPU restatement of openPSTD's PSTD solve (kernel/ and kernel/core/ of the
// openPSTD source tree), written from the reference's published algorithm and
// used only as the checker by tests/, by __graft_entry__.smoke() and by
// bench.py's CPU-baseline / reference arm.  Nothing in openpstd_gb300/ links or
// calls this file.
//
// Parity status: pinned by the reference's own known-answer tests
// (test/Kernel/kernel_functions.cpp, test/Kernel/WisdomCache.cpp,
// test/Kernel/Domain.cpp, test/Kernel/Scene.cpp); see tests/test_oracle_kats.py.
// The reference itself cannot be built here (Eigen, FFTW3f, Boost and Qt5 are
// absent), so end-to-end solves are pinned only through this restatement.
//
// The real FFT is the project's own (radix-2 complex FFT of half length with
// double-precision twiddles), not FFTW 3.3.5; FFTW's exact rounding is
// therefore not reproduced.  The c2r follows FFTW's convention of ignoring the
// imaginary parts of the DC and Nyquist bins and of not normalising.
//
// Template parameter T selects the arithmetic: float restates the reference
// build; double is the FP64 oracle.  Scene geometry (world->grid scaling,
// neighbour detection, PML placement) is always evaluated in float, as the
// reference does (QVector2D is float), so both instances share one topology.
//
// Quirks reproduced on purpose (the reference's CPU PSTDKernel is the parity
// target):
//   * y-direction neighbours are passed as (bottom, top) to the strip
//     derivative (kernel/core/Domain.cpp:104-107);
//   * edge parameters T and B are swapped (kernel/PSTDKernel.cpp:181-190);
//   * y-PML attenuation orientation (kernel/core/Domain.cpp:680-685,764-777);
//   * p0 is not recomputed after the PML multiply (kernel/Solver.cpp:85,114-116);
//   * receivers read p0(rel.x, rel.y) with rows = y (kernel/core/Receiver.cpp:80-83);
//   * the combination loop of Domain::calc writes the contiguous span
//     [min, max] of every clipped range (kernel/core/Domain.cpp:185-189,348,368);
//   * derivative arrays of directions with should_update == false keep their
//     previous (initially zero) content (kernel/Solver.cpp:101-104);
//   * has_horizontal_attenuation is read before it is assigned
//     (kernel/core/Domain.cpp:591-595 vs 657,684): taken as false.
// Cases where the reference reads undefined memory are rejected with an error
// instead of being emulated: more than one vacant run on an edge
// (kernel/core/Domain.cpp:570-583 writes row 0 only), a neighbour narrower than
// the window, a clipped range outside a neighbour's rows, a transform length
// that disagrees with the derivative-factor length
// (kernel/core/Domain.cpp:196-205 vs kernel/core/kernel_functions.cpp:166),
// and receiver indices outside p0 after the transposed lookup.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/pstd_gb300.h"

namespace orc {

static thread_local std::string g_err;

struct OracleError : std::runtime_error {
    int code;
    OracleError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum Direction { LEFT = 0, RIGHT = 1, TOP = 2, BOTTOM = 3 };      // kernel/core/kernel_functions.h:80-82
enum CalcDirection { CX = 0, CY = 1 };
enum CalcType { PRESSURE = 0, VELOCITY = 1 };
static const Direction all_directions[4] = {LEFT, RIGHT, TOP, BOTTOM};
static const float EPSILON = 1E-5f;                                 // kernel/core/kernel_functions.h:65
static const float rk_coefficients_ref[6] = {1.179799016570605e-1f, 1.846469664911166e-1f,
                                             2.466236043095944e-1f, 3.318395427360000e-1f, 5e-1f, 1.f};

static Direction opposite(Direction d) {
    switch (d) { case TOP: return BOTTOM; case BOTTOM: return TOP; case LEFT: return RIGHT; default: return LEFT; }
}
static CalcDirection dir_to_cd(Direction d) { return (d == LEFT || d == RIGHT) ? CX : CY; }

// ---------------------------------------------------------------- helpers
// kernel/core/kernel_functions.cpp:66-72
static int next_2_power(double n) {
    return std::max((int)std::pow(2.0, std::ceil(std::log2(n))), 1);
}
// kernel/core/WisdomCache.cpp:113-115
static int match_number(int n) { return (int)std::ceil(std::log2((double)n)); }

// kernel/KernelInterface.cpp:128-134
static int window_size(float patcherror) {
    int tmp = (int)std::round((patcherror * 0.7 - 17) / 2.);
    tmp = (int)std::round(tmp * 2);
    return tmp;
}

// kernel/core/kernel_functions.cpp:327-333 ; 2W+1 coefficients
template <class T>
static std::vector<T> window_coefficients(int W, int patch_error) {
    T window_alpha = (T)((patch_error - 40) / 20.0 + 1);
    T ln10 = (T)std::log(10.0);
    std::vector<T> w(2 * W + 1);
    T step = (T)(2 * W) / (T)(2 * W);   // LinSpaced(2W+1, -W, W): step (high-low)/(n-1)
    for (int i = 0; i < 2 * W + 1; i++) {
        T lin = (T)(-W) + (T)i * step;
        T x = lin / (T)W;
        T x2 = x * x;
        T x6 = x2 * x2 * x2;
        w[i] = std::exp(x6 * ln10 * window_alpha * (T)-1);
    }
    return w;
}

template <class T>
struct RhoArray { T pressure[4][2]; T velocity[4][2]; };

// kernel/core/kernel_functions.cpp:37-64
template <class T>
static RhoArray<T> get_rho_array(T rho1, T rho_self, T rho2) {
    T zn1 = rho1 / rho_self, inv_zn1 = rho_self / rho1;
    T rlw1 = (zn1 - 1) / (zn1 + 1), rlw2 = (inv_zn1 - 1) / (inv_zn1 + 1);
    T tlw1 = (2 * zn1) / (zn1 + 1), tlw2 = (2 * inv_zn1) / (inv_zn1 + 1);
    T zn2 = rho2 / rho_self, inv_zn2 = rho_self / rho2;
    T rrw1 = (zn2 - 1) / (zn2 + 1), rrw2 = (inv_zn2 - 1) / (inv_zn2 + 1);
    T trw1 = (2 * zn2) / (zn2 + 1), trw2 = (2 * inv_zn2) / (inv_zn2 + 1);
    RhoArray<T> r;
    T p[4][2] = {{rlw1, rlw2}, {rrw1, rrw2}, {tlw1, tlw2}, {trw1, trw2}};
    T v[4][2] = {{-rlw1, -rlw2}, {-rrw1, -rrw2}, {tlw2, tlw1}, {trw2, trw1}};
    std::memcpy(r.pressure, p, sizeof p);
    std::memcpy(r.velocity, v, sizeof v);
    return r;
}

// kernel/core/WisdomCache.cpp:53-75 ; length 2^match_number(N)
template <class T>
struct Discretization {
    std::vector<T> wave_numbers;
    std::vector<std::complex<T>> complex_factors, pressure_deriv_factors, velocity_deriv_factors;
};

template <class T>
static Discretization<T> discretize_wave_numbers(T dx, int matched) {
    T max_wave_number = (T)M_PI / dx;
    int two_power = (int)std::pow(2.0, matched - 1);
    T dka = max_wave_number / (T)two_power;
    Discretization<T> d;
    int n = 2 * two_power;
    d.wave_numbers.resize(n);
    {   // head: LinSpaced(two_power+1, 0, max)
        T step = (max_wave_number - 0) / (T)(two_power);
        for (int i = 0; i <= two_power; i++) d.wave_numbers[i] = (T)0 + (T)i * step;
    }
    if (two_power - 1 > 0) {  // tail: LinSpaced(two_power-1, max-dka, dka)
        int m = two_power - 1;
        T lo = max_wave_number - dka, hi = dka;
        T step = (m > 1) ? (hi - lo) / (T)(m - 1) : (T)0;
        for (int i = 0; i < m; i++) d.wave_numbers[two_power + 1 + i] = (m > 1) ? lo + (T)i * step : hi;
    }
    d.complex_factors.resize(n);
    d.pressure_deriv_factors.resize(n);
    d.velocity_deriv_factors.resize(n);
    T half = (T)(dx * (T)0.5);
    for (int i = 0; i < n; i++) {
        T im = (i < two_power + 1) ? (T)1 : (T)-1;
        d.complex_factors[i] = std::complex<T>(0, im);
        std::complex<T> ck = d.complex_factors[i] * d.wave_numbers[i];
        d.pressure_deriv_factors[i] = std::exp(-ck * half) * ck;
        d.velocity_deriv_factors[i] = std::exp(ck * half) * ck;
    }
    return d;
}

// ---------------------------------------------------------------- real FFT
// Own implementation: complex radix-2 FFT of length L/2 with twiddles built
// in double precision, plus the standard even/odd split for r2c and c2r.
template <class T>
struct RealFFT {
    int L = 0, H = 0;
    std::vector<std::complex<T>> tw_half;   // exp(-2 pi i j / H), j < H/2
    std::vector<std::complex<T>> tw_full;   // exp(-2 pi i k / L), k <= H
    std::vector<int> bitrev;
    explicit RealFFT(int L_) : L(L_), H(L_ / 2) {
        tw_half.resize(std::max(1, H / 2));
        for (int j = 0; j < H / 2; j++) {
            double a = -2.0 * M_PI * j / H;
            tw_half[j] = std::complex<T>((T)std::cos(a), (T)std::sin(a));
        }
        tw_full.resize(H + 1);
        for (int k = 0; k <= H; k++) {
            double a = -2.0 * M_PI * k / L;
            tw_full[k] = std::complex<T>((T)std::cos(a), (T)std::sin(a));
        }
        bitrev.resize(H);
        int bits = 0;
        while ((1 << bits) < H) bits++;
        for (int i = 0; i < H; i++) {
            int r = 0;
            for (int b = 0; b < bits; b++) if (i & (1 << b)) r |= 1 << (bits - 1 - b);
            bitrev[i] = r;
        }
    }
    // in-place complex FFT of length H; inverse uses conjugate twiddles, unnormalised
    void cfft(std::complex<T>* z, bool inverse) const {
        for (int i = 0; i < H; i++) if (i < bitrev[i]) std::swap(z[i], z[bitrev[i]]);
        for (int len = 2; len <= H; len <<= 1) {
            int half = len >> 1, step = H / len;
            for (int s = 0; s < H; s += len) {
                for (int j = 0; j < half; j++) {
                    std::complex<T> w = tw_half[j * step];
                    if (inverse) w = std::conj(w);
                    std::complex<T> a = z[s + j], b = z[s + j + half] * w;
                    z[s + j] = a + b;
                    z[s + j + half] = a - b;
                }
            }
        }
    }
    // r2c: x[L] -> X[H+1]
    void r2c(const T* x, std::complex<T>* X, std::complex<T>* work) const {
        for (int n = 0; n < H; n++) work[n] = std::complex<T>(x[2 * n], x[2 * n + 1]);
        cfft(work, false);
        const std::complex<T> mi(0, -1);
        for (int k = 0; k <= H; k++) {
            std::complex<T> a = work[k % H], b = std::conj(work[(H - k) % H]);
            std::complex<T> E = (a + b) * (T)0.5, O = (a - b) * (T)0.5 * mi;
            X[k] = E + tw_full[k] * O;
        }
    }
    // c2r (FFTW convention: unnormalised; imag of DC and Nyquist ignored)
    void c2r(std::complex<T>* X, T* x, std::complex<T>* work) const {
        X[0] = std::complex<T>(X[0].real(), 0);
        X[H] = std::complex<T>(X[H].real(), 0);
        const std::complex<T> pi(0, 1);
        for (int k = 0; k < H; k++) {
            std::complex<T> a = X[k], b = std::conj(X[H - k]);
            work[k] = (a + b) + pi * std::conj(tw_full[k]) * (a - b);
        }
        cfft(work, true);
        for (int n = 0; n < H; n++) { x[2 * n] = work[n].real(); x[2 * n + 1] = work[n].imag(); }
    }
};

template <class T>
static const RealFFT<T>& fft_plan(int L) {
    static thread_local std::map<int, std::unique_ptr<RealFFT<T>>> cache;
    auto it = cache.find(L);
    if (it != cache.end()) return *it->second;
    auto p = std::make_unique<RealFFT<T>>(L);
    auto& ref = *p;
    cache[L] = std::move(p);
    return ref;
}

// strip matrix: `batch` strips of length `n`, strip-major
template <class T>
struct Strips {
    int batch = 0, n = 0;
    std::vector<T> a;
    Strips() {}
    Strips(int b, int n_) : batch(b), n(n_), a((size_t)b * n_, (T)0) {}
    T& operator()(int s, int i) { return a[(size_t)s * n + i]; }
    T operator()(int s, int i) const { return a[(size_t)s * n + i]; }
};

// kernel/core/kernel_functions.cpp:123-318 (strips already laid out along the
// derivative direction, i.e. after the optional transpose of lines 154-159).
template <class T>
static Strips<T> spatderp3(const Strips<T>& p1, const Strips<T>& p2, const Strips<T>& p3,
                           const std::vector<std::complex<T>>& derfact, const RhoArray<T>& rho,
                           const std::vector<T>& window, int wlen, CalcType ct) {
    int batch = p2.batch;
    int n = p2.n;
    int L = next_2_power((double)(n + wlen * 2));
    if ((int)derfact.size() < L / 2 + 1)
        throw OracleError(PSTD_ERR_UNSUPPORTED, "derivative factors shorter than the transform (reference reads past derfact)");
    bool pres = (ct == PRESSURE);
    if (pres ? (wlen > p1.n || wlen > p3.n) : (wlen + 1 > p1.n || wlen + 1 > p3.n))
        throw OracleError(PSTD_ERR_UNSUPPORTED, "window wider than a neighbour strip (reference reads out of bounds)");
    const RealFFT<T>& plan = fft_plan<T>(L);
    int nout = pres ? n + 1 : n - 1;
    Strips<T> result(batch, nout);
    std::vector<T> buf(L);
    std::vector<std::complex<T>> spec(L / 2 + 1), work(L / 2 + 1);
    // window.head(wlen) / window.tail(wlen)
    const T* wl = window.data();
    const T* wr = window.data() + wlen + 1;
    T R1, T1, R2, T2;
    if (pres) { T1 = rho.pressure[2][1]; R1 = rho.pressure[0][0]; T2 = rho.pressure[3][1]; R2 = rho.pressure[1][0]; }
    else      { T1 = rho.velocity[2][1]; R1 = rho.velocity[0][0]; T2 = rho.velocity[3][1]; R2 = rho.velocity[1][0]; }
    for (int s = 0; s < batch; s++) {
        std::fill(buf.begin(), buf.end(), (T)0);
        int n1 = p1.n, n3 = p3.n;
        for (int j = 0; j < wlen; j++) {
            T a, b, c, d;
            if (pres) {
                a = p1(s, n1 - wlen + j);          // p1.rightCols(wlen)
                b = p2(s, wlen - 1 - j);           // p2.leftCols(wlen) reversed
                c = p3(s, j);                      // p3.leftCols(wlen)
                d = p2(s, n - 1 - j);              // p2.rightCols(wlen) reversed
            } else {
                a = p1(s, n1 - wlen - 1 + j);      // p1.rightCols(wlen+1).leftCols(wlen)
                b = p2(s, wlen - j);               // p2.leftCols(wlen+1).rightCols(wlen) reversed
                c = p3(s, 1 + j);                  // p3.leftCols(wlen+1).rightCols(wlen)
                d = p2(s, n - 2 - j);              // p2.rightCols(wlen+1).leftCols(wlen) reversed
            }
            T dom1 = a * T1 + b * R1;
            T dom3 = c * T2 + d * R2;
            buf[j] = dom1 * wl[j];
            buf[wlen + n + j] = dom3 * wr[j];
        }
        (void)n3;
        for (int i = 0; i < n; i++) buf[wlen + i] = p2(s, i);
        plan.r2c(buf.data(), spec.data(), work.data());
        for (int k = 0; k <= L / 2; k++) spec[k] = spec[k] * derfact[k];
        plan.c2r(spec.data(), buf.data(), work.data());
        for (int i = 0; i < nout; i++) result(s, i) = buf[wlen + i] / (T)L;
    }
    return result;
}

// ---------------------------------------------------------------- scene
struct Point { int x = 0, y = 0; };

struct EdgeParameters { bool locally_reacting = false; float alpha = 0; };

template <class T>
struct Field2 {   // Eigen-shaped (rows = y, cols = x), stored row-major
    int rows = 0, cols = 0;
    std::vector<T> a;
    void zeros(int r, int c) { rows = r; cols = c; a.assign((size_t)r * c, (T)0); }
    T& operator()(int r, int c) { return a[(size_t)r * cols + c]; }
    T operator()(int r, int c) const { return a[(size_t)r * cols + c]; }
};

template <class T>
struct Domain {
    int id = 0;
    float alpha = 0;
    T impedance = 0, rho = 0;
    bool rigid = false;
    Point top_left, size, bottom_right;
    bool is_pml = false, is_secondary_pml = false, local = false;
    std::vector<Domain*> pml_for_domain_list;
    std::map<Direction, EdgeParameters> edge_param_map;
    bool should_update[2] = {true, true};
    std::vector<Domain*> left, right, top, bottom;
    int num_neighbour_domains = 0, num_pml_neighbour_domains = 0;
    bool has_horizontal_attenuation = false;   // Q8 convention: value-initialised
    bool is_corner_domain = false;
    std::vector<bool> needs_reversed_attenuation;
    // fields
    Field2<T> p0, px0, py0, vx0, vy0;            // current
    Field2<T> pp0, ppx0, ppy0, pvx0, pvy0;       // previous
    Field2<T> Lpx, Lpy, Lvx, Lvy;
    Field2<T> pml_px, pml_py, pml_vx, pml_vy;

    std::vector<Domain*>& nb(Direction d) {
        switch (d) { case LEFT: return left; case RIGHT: return right; case TOP: return top; default: return bottom; }
    }
    // kernel/core/Domain.cpp:435-448
    std::vector<int> get_range(CalcDirection cd) const {
        int a = (cd == CX) ? top_left.y : top_left.x;
        int b = (cd == CX) ? bottom_right.y : bottom_right.x;
        std::vector<int> r(std::max(0, b - a));
        std::iota(r.begin(), r.end(), a);
        return r;
    }
    bool is_neighbour_of(Domain* o) {
        for (Direction d : all_directions) {
            auto& v = nb(d);
            if (std::find(v.begin(), v.end(), o) != v.end()) return true;
        }
        return false;
    }
    bool is_pml_for(Domain* o) {
        return std::find(pml_for_domain_list.begin(), pml_for_domain_list.end(), o) != pml_for_domain_list.end();
    }
    int number_of_neighbours(bool count_pml) {
        return count_pml ? num_neighbour_domains : num_neighbour_domains - num_pml_neighbour_domains;
    }
    int get_num_pmls_in_direction(Direction d) {
        int n = 0;
        for (auto* o : nb(d)) if (o->is_pml) n++;
        return n;
    }
    bool contains_location(const float loc[3]) const {
        int tl[3] = {top_left.x, top_left.y, 0};
        int br[3] = {bottom_right.x, bottom_right.y, 0};
        for (int d = 0; d < 3; d++) if ((float)tl[d] > loc[d] || loc[d] > (float)br[d]) return false;
        return true;
    }
};

struct SettingsF {
    float calctime, c1, ampMax, rho, patcherror, tfactRK, dx, band_width;
    float rk[6];
    int pml_cells, save_nth;
    float time_step() const { return tfactRK * dx / c1; }          // kernel/KernelInterface.cpp:125-127
    int window() const { return window_size(patcherror); }
};

template <class T>
struct Receiver {
    int id;
    Point grid;
    Domain<T>* container;
    float gx = 0, gy = 0;   // grid location (spectral receivers)
};

template <class T>
struct Scene {
    SettingsF s;
    std::vector<std::unique_ptr<Domain<T>>> owned;
    std::vector<Domain<T>*> domain_list;
    std::vector<Receiver<T>> receivers;
    bool spectral = false;   // settings.spectral_interpolation == PSTD_RECEIVERS_SPECTRAL
    int number_of_domains = 0;
    int framecount = 0;
    std::map<int, Discretization<T>> disc_cache;

    int get_new_id() { return number_of_domains++; }

    Domain<T>* make_domain(int id, float alpha, Point tl, Point sz, bool is_pml, Domain<T>* pml_for) {
        auto d = std::make_unique<Domain<T>>();
        Domain<T>* p = d.get();
        owned.push_back(std::move(d));
        // kernel/core/Domain.cpp:53-92
        p->id = id;
        p->alpha = alpha;
        p->top_left = tl;
        p->size = sz;
        p->bottom_right = Point{tl.x + sz.x, tl.y + sz.y};
        float sa = std::sqrt(1.0f - alpha);
        float impf = -((sa + 1) / (sa - 1));
        p->rigid = impf > 1000;                                     // kernel/core/Domain.cpp:431-433
        T sat = std::sqrt((T)1 - (T)alpha);
        p->impedance = -((sat + 1) / (sat - 1));
        p->rho = p->rigid ? (T)1E30 : (T)s.rho * p->impedance;
        if (is_pml) p->pml_for_domain_list.push_back(pml_for);
        p->is_pml = is_pml;
        p->is_secondary_pml = false;
        for (auto* o : p->pml_for_domain_list) if (o->is_pml) p->is_secondary_pml = true;
        p->p0.zeros(sz.y, sz.x); p->px0.zeros(sz.y, sz.x); p->py0.zeros(sz.y, sz.x);
        p->vx0.zeros(sz.y, sz.x + 1); p->vy0.zeros(sz.y + 1, sz.x);
        p->Lpx.zeros(sz.y, sz.x + 1); p->Lpy.zeros(sz.y + 1, sz.x);
        p->Lvx.zeros(sz.y, sz.x); p->Lvy.zeros(sz.y, sz.x);
        p->pml_px.zeros(sz.y, sz.x); p->pml_py.zeros(sz.y, sz.x);
        p->pml_vx.zeros(sz.y, sz.x + 1); p->pml_vy.zeros(sz.y + 1, sz.x);
        p->local = false;
        return p;
    }

    // kernel/core/Scene.cpp:297-380
    void add_domain(Domain<T>* domain) {
        for (size_t i = 0; i < domain_list.size(); i++) {
            Domain<T>* other = domain_list[i];
            if (domain->is_secondary_pml && other->is_secondary_pml) continue;
            if ((domain->is_secondary_pml && !other->is_pml) || (other->is_secondary_pml && !domain->is_pml)) continue;
            if (domain->is_pml && other->is_pml) {
                bool pml_for_domain = other->is_pml_for(domain);
                bool pml_for_other = domain->is_pml_for(other);
                if ((domain->is_secondary_pml && pml_for_other) || (other->is_secondary_pml && pml_for_domain)) {
                } else if (other->pml_for_domain_list.size() != 1 || domain->pml_for_domain_list.size() != 1) {
                    continue;
                } else if (!other->pml_for_domain_list[0]->is_neighbour_of(domain->pml_for_domain_list[0])) {
                    continue;
                } else if (!domain->pml_for_domain_list[0]->is_neighbour_of(other->pml_for_domain_list[0])) {
                    continue;
                }
            }
            Direction orientation = LEFT;
            bool is_neighbour = true;
            if (domain->bottom_right.x == other->top_left.x) orientation = RIGHT;
            else if (domain->top_left.x == other->bottom_right.x) orientation = LEFT;
            else if (domain->bottom_right.y == other->top_left.y) orientation = BOTTOM;
            else if (domain->top_left.y == other->bottom_right.y) orientation = TOP;
            else is_neighbour = false;
            bool other_pml_for_different = other->is_pml && !domain->is_pml && !other->is_pml_for(domain);
            bool domain_pml_for_different = domain->is_pml && !other->is_pml && !domain->is_pml_for(other);
            if (is_neighbour && !other_pml_for_different && !domain_pml_for_different) {
                CalcDirection cd = dir_to_cd(orientation);
                auto a = domain->get_range(cd), b = other->get_range(cd);
                std::vector<int> inter;
                std::set_intersection(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(inter));
                if (!inter.empty()) {
                    domain->nb(orientation).push_back(other);
                    other->nb(opposite(orientation)).push_back(domain);
                }
            }
        }
        domain_list.push_back(domain);
    }

    // kernel/core/Domain.cpp:543-584 ; single-run edges only
    std::vector<std::pair<int, int>> get_vacant_range(Domain<T>* d, Direction dir) {
        CalcDirection cd = dir_to_cd(dir);
        auto range = d->get_range(cd);
        std::set<int> rs(range.begin(), range.end());
        for (auto* o : d->nb(dir)) {
            auto nr = o->get_range(cd);
            for (int v : nr) rs.erase(v);
        }
        std::vector<int> r(rs.begin(), rs.end());
        std::vector<std::pair<int, int>> runs;
        for (size_t i = 0; i < r.size(); i++) {
            if (i == 0 || r[i - 1] + 1 < r[i]) runs.push_back({r[i], r[i]});
            if (i == r.size() - 1 || r[i + 1] - 1 > r[i]) runs.back().second = r[i] + 1;
        }
        if (runs.size() > 1)
            throw OracleError(PSTD_ERR_UNSUPPORTED,
                              "edge with more than one vacant run (reference get_vacant_range leaves rows uninitialised)");
        return runs;
    }

    // kernel/core/Scene.cpp:41-225
    void add_pml_domains() {
        int P = s.pml_cells;
        const Direction directions[4] = {LEFT, TOP, RIGHT, BOTTOM};
        std::vector<Domain<T>*> first_order;
        std::vector<std::pair<Domain<T>*, Direction>> second_order;   // creation order (reference: pointer order)
        std::vector<Domain<T>*> snapshot = domain_list;
        for (auto* domain : snapshot) {
            if (domain->is_pml) continue;
            for (int i = 0; i < 4; i++) {
                Direction direction = directions[i];
                auto vac = get_vacant_range(domain, direction);
                for (auto& run : vac) {
                    int pml_id = get_new_id();
                    float alpha = domain->edge_param_map[direction].alpha;
                    float pml_alpha = std::max(alpha, EPSILON);
                    int xo = 0, yo = 0, xs = 0, ys = 0;
                    switch (direction) {
                        case LEFT: xo = -P; yo = run.first - domain->top_left.y; xs = P; ys = run.second - run.first; break;
                        case RIGHT: xo = domain->size.x; yo = run.first - domain->top_left.y; xs = P; ys = run.second - run.first; break;
                        case TOP: xo = run.first - domain->top_left.x; yo = -P; xs = run.second - run.first; ys = P; break;
                        case BOTTOM: xo = run.first - domain->top_left.x; yo = domain->size.y; xs = run.second - run.first; ys = P; break;
                    }
                    Point tl{domain->top_left.x + xo, domain->top_left.y + yo};
                    bool full_overlap = (dir_to_cd(direction) == CX)
                        ? (run.first == domain->top_left.y && run.second == domain->bottom_right.y)
                        : (run.first == domain->top_left.x && run.second == domain->bottom_right.x);
                    Domain<T>* pml = make_domain(pml_id, pml_alpha, tl, Point{xs, ys}, true, domain);
                    first_order.push_back(pml);
                    if (!full_overlap) pml->local = true;
                    if (alpha > 0 && full_overlap) {
                        int dirs2[2] = {(i + 1) % 4, (i + 3) % 4};
                        for (int k = 0; k < 2; k++) {
                            Direction second_dir = directions[dirs2[k]];
                            int sid = get_new_id();
                            float other_alpha = domain->edge_param_map[second_dir].alpha;
                            float sa = std::min(std::max(EPSILON, other_alpha), std::max(EPSILON, pml_alpha));
                            int sx = 0, sy = 0;
                            switch (second_dir) {
                                case LEFT: sx = -P; sy = 0; break;
                                case RIGHT: sx = pml->size.x; sy = 0; break;
                                case TOP: sx = 0; sy = -P; break;
                                case BOTTOM: sx = 0; sy = pml->size.y; break;
                            }
                            Point stl{domain->top_left.x + xo + sx, domain->top_left.y + yo + sy};
                            Domain<T>* sec = make_domain(sid, sa, stl, Point{P, P}, true, pml);
                            second_order.push_back({sec, second_dir});
                        }
                    }
                }
            }
        }
        for (auto* d : first_order) add_domain(d);
        std::map<std::vector<int>, std::vector<Domain<T>*>> by_corner;
        for (auto& e : second_order) {
            Domain<T>* parent = e.first->pml_for_domain_list.at(0);
            if (!parent->nb(e.second).empty()) continue;
            std::vector<int> key = {e.first->top_left.x, e.first->top_left.y, e.first->bottom_right.x, e.first->bottom_right.y};
            by_corner[key].push_back(e.first);
        }
        auto singular_parent = [](Domain<T>* d) -> Domain<T>* {
            if (d != nullptr && d->is_pml && d->pml_for_domain_list.size() == 1) return d->pml_for_domain_list[0];
            return nullptr;
        };
        std::vector<Domain<T>*> second_list;
        for (auto& e : by_corner) {
            auto& v = e.second;
            if (v.size() == 1) { second_list.push_back(v[0]); continue; }
            std::vector<Domain<T>*> processed;
            for (size_t i = 0; i < v.size(); i++) {
                for (size_t j = i + 1; j < v.size(); j++) {
                    Domain<T>* di = v[i]; Domain<T>* dj = v[j];
                    bool pi = std::find(processed.begin(), processed.end(), di) != processed.end();
                    bool pj = std::find(processed.begin(), processed.end(), dj) != processed.end();
                    if (pi || pj) continue;
                    Domain<T>* g1 = singular_parent(singular_parent(di));
                    Domain<T>* g2 = singular_parent(singular_parent(dj));
                    if (g1 != nullptr && g2 != nullptr && g1->id == g2->id) {
                        processed.push_back(di); processed.push_back(dj);
                        for (auto* pf : dj->pml_for_domain_list) di->pml_for_domain_list.push_back(pf);
                        second_list.push_back(di);
                    }
                }
            }
            for (auto* d : v) if (std::find(processed.begin(), processed.end(), d) == processed.end()) second_list.push_back(d);
        }
        for (auto* d : second_list) add_domain(d);
    }

    // kernel/core/Domain.cpp:504-515,587-616,787-790
    void post_initialization(Domain<T>* d) {
        d->num_neighbour_domains = 0; d->num_pml_neighbour_domains = 0;
        for (Direction dir : all_directions)
            for (auto* o : d->nb(dir)) { d->num_neighbour_domains++; if (o->is_pml) d->num_pml_neighbour_domains++; }
        for (int cdi = 0; cdi < 2; cdi++) {
            CalcDirection cd = (CalcDirection)cdi;
            bool su = true;
            if (d->number_of_neighbours(false) == 1 && d->is_pml) {
                if (d->has_horizontal_attenuation && cd == CX) su = true;
                else if (!d->has_horizontal_attenuation && cd == CY) su = true;
                else if (d->local) su = false;
                else {
                    for (Direction dir : all_directions) {
                        auto& dn = d->nb(dir);
                        if (dn.size() == 1 && !dn[0]->is_pml) su = !dn[0]->edge_param_map[dir].locally_reacting;
                    }
                }
            }
            d->should_update[cdi] = su;
        }
    }

    // kernel/core/Domain.cpp:743-780
    void create_attenuation_array(Domain<T>* d, CalcDirection cd, bool ascending, Field2<T>& fp, Field2<T>& fv) {
        int P = s.pml_cells;
        T dt = (T)s.time_step();
        std::vector<T> pf(P), vf(P + 1);
        T pstep = (T)((float)P - 0.5f - 0.5f) / (T)(P - 1 > 0 ? P - 1 : 1);
        for (int i = 0; i < P; i++) {
            T r = (P > 1 ? (T)0.5 + (T)i * pstep : (T)0.5) / (T)P;
            T r4 = std::pow(r, (T)4);
            T ap = (T)s.ampMax * r4;
            pf[i] = std::exp(-ap * dt / (T)s.rho);
        }
        T vstep = (T)P / (T)P;
        for (int i = 0; i <= P; i++) {
            T r = ((T)0 + (T)i * vstep) / (T)P;
            T r4 = std::pow(r, (T)4);
            T av = (T)s.rho * (T)s.ampMax * r4;
            vf[i] = std::exp(-av * dt);
        }
        if (!ascending) { std::reverse(pf.begin(), pf.end()); std::reverse(vf.begin(), vf.end()); }
        if (cd == CX) {
            if (d->size.x != P) throw OracleError(PSTD_ERR_UNSUPPORTED, "PML attenuation profile does not match domain width");
            fp.zeros(d->size.y, P); fv.zeros(d->size.y, P + 1);
            for (int r = 0; r < d->size.y; r++) {
                for (int c = 0; c < P; c++) fp(r, c) = pf[c];
                for (int c = 0; c <= P; c++) fv(r, c) = vf[c];
            }
        } else {
            if (d->size.y != P) throw OracleError(PSTD_ERR_UNSUPPORTED, "PML attenuation profile does not match domain height");
            fp.zeros(P, d->size.x); fv.zeros(P + 1, d->size.x);
            for (int r = 0; r < P; r++) for (int c = 0; c < d->size.x; c++) fp(r, c) = pf[r];
            for (int r = 0; r <= P; r++) for (int c = 0; c < d->size.x; c++) fv(r, c) = vf[r];
        }
    }

    static void fill_ones(Field2<T>& f, int r, int c) { f.rows = r; f.cols = c; f.a.assign((size_t)r * c, (T)1); }

    // kernel/core/Domain.cpp:644-714
    void compute_pml_matrices(Domain<T>* d) {
        int n_normal = d->num_neighbour_domains - d->num_pml_neighbour_domains;
        (void)n_normal;
        if (d->is_secondary_pml) {
            d->is_corner_domain = d->num_neighbour_domains == 2;
            d->has_horizontal_attenuation = !d->left.empty() || !d->right.empty();
            if (d->is_corner_domain) {
                if (!(d->has_horizontal_attenuation && (!d->top.empty() || !d->bottom.empty())))
                    throw OracleError(PSTD_ERR_UNSUPPORTED, "corner PML without horizontal and vertical neighbour");
                d->needs_reversed_attenuation.clear();
                d->needs_reversed_attenuation.push_back(!d->left.empty());
                d->needs_reversed_attenuation.push_back(!d->bottom.empty());
            } else {
                d->needs_reversed_attenuation.push_back(!d->left.empty() || !d->bottom.empty());
            }
        } else {
            d->is_corner_domain = false;
            bool all_air_left = !d->left.empty() && d->get_num_pmls_in_direction(LEFT) == 0;
            bool all_air_right = !d->right.empty() && d->get_num_pmls_in_direction(RIGHT) == 0;
            bool all_air_bottom = !d->bottom.empty() && d->get_num_pmls_in_direction(BOTTOM) == 0;
            d->has_horizontal_attenuation = all_air_left || all_air_right;
            d->needs_reversed_attenuation.push_back(all_air_left || all_air_bottom);
        }
        if (d->is_secondary_pml && d->is_corner_domain) {
            create_attenuation_array(d, CX, d->needs_reversed_attenuation.at(0), d->pml_px, d->pml_vx);
            create_attenuation_array(d, CY, d->needs_reversed_attenuation.at(1), d->pml_py, d->pml_vy);
        } else if (d->has_horizontal_attenuation) {
            create_attenuation_array(d, CX, d->needs_reversed_attenuation.at(0), d->pml_px, d->pml_vx);
            fill_ones(d->pml_py, d->size.y, d->size.x);
            fill_ones(d->pml_vy, d->size.y + 1, d->size.x);
        } else {
            create_attenuation_array(d, CY, d->needs_reversed_attenuation.at(0), d->pml_py, d->pml_vy);
            fill_ones(d->pml_px, d->size.y, d->size.x);
            fill_ones(d->pml_vx, d->size.y, d->size.x + 1);
        }
    }

    // kernel/core/Speaker.cpp:21-39, kernel/core/Scene.cpp:267-279
    void add_speaker(float gx, float gy) {
        float x = gx - 0.5f, y = gy - 0.5f;
        for (auto* d : domain_list) {
            T dx = (T)s.dx;
            T rel_x = (T)(x - (float)d->top_left.x);
            T rel_y = (T)(y - (float)d->top_left.y);
            for (int i = 0; i < d->size.x; i++) {
                for (int j = 0; j < d->size.y; j++) {
                    // SQR(a) expands to a*a without parentheses: ((rel-i)*dx*(rel-i))*dx
                    T sq = (rel_x - (T)i) * dx * (rel_x - (T)i) * dx + (rel_y - (T)j) * dx * (rel_y - (T)j) * dx;
                    T pressure = std::exp(-(T)s.band_width * sq);
                    T angle = std::atan2(rel_x - (T)i, rel_y - (T)j);
                    T h = std::cos(angle) * std::cos(angle) * pressure;
                    T v = std::sin(angle) * std::sin(angle) * pressure;
                    d->p0(j, i) += pressure;
                    d->px0(j, i) += h;
                    d->py0(j, i) += v;
                }
            }
        }
    }

    // kernel/core/Scene.cpp:254-265, kernel/core/Receiver.cpp:34-44
    void add_receiver(float x, float y, int id) {
        float loc[3] = {x, y, 0.f};
        Domain<T>* container = nullptr;
        for (auto* d : domain_list) if (!d->is_pml && d->contains_location(loc)) container = d;
        if (!container) throw OracleError(PSTD_ERR_INVALID, "receiver outside every non-PML domain");
        Receiver<T> r;
        r.id = id;
        r.grid = Point{(int)x, (int)y};
        r.container = container;
        r.gx = x;
        r.gy = y;
        int rx = r.grid.x - container->top_left.x, ry = r.grid.y - container->top_left.y;
        if (spectral) {
            // the point lies in cell (rx, ry) of the container (x offset rx)
            if (rx < 0 || ry < 0 || rx >= container->size.x || ry >= container->size.y)
                throw OracleError(PSTD_ERR_UNSUPPORTED, "spectral receiver on the far edge of its domain");
        } else if (rx < 0 || ry < 0 || rx >= container->size.y || ry >= container->size.x) {
            // p0(rel.x, rel.y): row index rel.x must be < Ny, column rel.y < Nx
            throw OracleError(PSTD_ERR_UNSUPPORTED, "receiver index outside p0 after the reference's transposed lookup");
        }
        receivers.push_back(r);
    }

    // kernel/core/WisdomCache.cpp:39-50 (std::map nodes stay valid after insert)
    const Discretization<T>& get_discretization(int N) {
        int m = match_number(N);
        const Discretization<T>* res = nullptr;
#pragma omp critical(orc_disc_cache)
        {
            auto it = disc_cache.find(m);
            if (it == disc_cache.end()) it = disc_cache.emplace(m, discretize_wave_numbers<T>((T)s.dx, m)).first;
            res = &it->second;
        }
        return *res;
    }

    // ------------------------------------------------------------ build
    void build(const pstd_config* cfg) {
        const pstd_settings& st = cfg->settings;
        s.calctime = st.calctime; s.c1 = st.c1; s.ampMax = st.ampMax; s.rho = st.rho;
        s.patcherror = st.patcherror; s.tfactRK = st.tfactRK; s.dx = st.gridSpacing;
        s.band_width = st.band_width; s.pml_cells = st.PMLCells; s.save_nth = st.SaveNth;
        if (st.n_rk_coefficients != 6) throw OracleError(PSTD_ERR_INVALID, "need 6 RK coefficients");
        for (int i = 0; i < 6; i++) s.rk[i] = st.rk_coefficients[i];
        spectral = st.spectral_interpolation == PSTD_RECEIVERS_SPECTRAL;
        if (s.dx <= 0 || s.c1 <= 0 || s.tfactRK <= 0) throw OracleError(PSTD_ERR_INVALID, "bad settings");
        // kernel/PSTDKernel.cpp:73-98,170-190
        std::vector<Domain<T>*> domains;
        for (int i = 0; i < cfg->n_domains; i++) {
            const pstd_domain_conf& dc = cfg->domains[i];
            float tlx = dc.top_left[0] / s.dx, tly = dc.top_left[1] / s.dx;
            float szx = dc.size[0] / s.dx, szy = dc.size[1] / s.dx;
            Point tl{(int)tlx, (int)tly}, sz{(int)szx, (int)szy};
            if (sz.x <= 0 || sz.y <= 0) throw OracleError(PSTD_ERR_INVALID, "empty domain");
            int id = get_new_id();
            Domain<T>* d = make_domain(id, 1.f, tl, sz, false, nullptr);
            d->edge_param_map[LEFT] = {dc.L.lr != 0, dc.L.absorption};
            d->edge_param_map[RIGHT] = {dc.R.lr != 0, dc.R.absorption};
            d->edge_param_map[TOP] = {dc.B.lr != 0, dc.B.absorption};
            d->edge_param_map[BOTTOM] = {dc.T.lr != 0, dc.T.absorption};
            domains.push_back(d);
        }
        for (auto* d : domains) add_domain(d);
        add_pml_domains();
        for (auto* d : domain_list) post_initialization(d);
        for (int i = 0; i < cfg->n_speakers; i++)
            add_speaker(cfg->speakers[3 * i] / s.dx, cfg->speakers[3 * i + 1] / s.dx);
        for (int i = 0; i < cfg->n_receivers; i++)
            add_receiver(cfg->receivers[3 * i] / s.dx, cfg->receivers[3 * i + 1] / s.dx, i);
        for (auto* d : domain_list) if (d->is_pml) compute_pml_matrices(d);
        framecount = (int)(s.calctime / s.time_step());      // kernel/Solver.cpp:41
    }

    // ------------------------------------------------------------ calc
    // kernel/core/Domain.cpp:95-391
    // shift != nullptr: the pressure strips are shifted by *shift cells
    // (factors exp(i k shift dx) in place of the derivative factors) into
    // *dest -- the spectral receivers' passes
    void calc(Domain<T>* self, CalcDirection cd, CalcType ct, const double* shift = nullptr,
              Field2<T>* dest = nullptr) {
        std::vector<int> own_range = self->get_range(cd);
        std::vector<Domain<T>*> domains1 = (cd == CX) ? self->left : self->bottom;
        std::vector<Domain<T>*> domains2 = (cd == CX) ? self->right : self->top;
        Field2<T>& source = dest ? *dest
                          : (ct == PRESSURE) ? (cd == CX ? self->Lpx : self->Lpy) : (cd == CX ? self->Lvx : self->Lvy);
        for (size_t i = 0; i != domains1.size() + 1; i++) {
            Domain<T>* d1 = (i != domains1.size()) ? domains1[i] : nullptr;
            for (size_t j = 0; j != domains2.size() + 1; j++) {
                Domain<T>* d2 = (j != domains2.size()) ? domains2[j] : nullptr;
                std::vector<int> inter = own_range;
                if (d1) {
                    auto r1 = d1->get_range(cd); std::vector<int> t;
                    std::set_intersection(r1.begin(), r1.end(), inter.begin(), inter.end(), std::back_inserter(t));
                    inter = t;
                }
                if (d2) {
                    auto r2 = d2->get_range(cd); std::vector<int> t;
                    std::set_intersection(r2.begin(), r2.end(), inter.begin(), inter.end(), std::back_inserter(t));
                    inter = t;
                }
                if (inter.empty()) continue;
                {
                    std::vector<int> diff;
                    std::set_difference(own_range.begin(), own_range.end(), inter.begin(), inter.end(),
                                        std::inserter(diff, diff.begin()));
                    own_range = diff;
                }
                int range_start = *std::min_element(inter.begin(), inter.end());
                int range_end = *std::max_element(inter.begin(), inter.end()) + 1;
                int primary_dimension = (cd == CX) ? self->size.x : self->size.y;
                int wlen = s.window();
                while (wlen > primary_dimension) wlen = wlen / 2;
                int N_total = 2 * wlen + primary_dimension;
                std::vector<T> wind = window_coefficients<T>(wlen, (int)s.patcherror);
                if (ct == PRESSURE) N_total++;
                bool side1_zero = false, side2_zero = false;
                if (!d1) { d1 = self; side1_zero = true; }
                if (!d2) { d2 = self; side2_zero = true; }
                const Discretization<T>& disc = get_discretization(N_total);
                std::vector<std::complex<T>> shift_factors;
                if (shift) {
                    // exp(i k shift dx) with k dx = 2 pi j / L for the bins j <= L/2 the transform uses
                    const int Ls = (int)disc.pressure_deriv_factors.size();
                    shift_factors.resize(Ls);
                    for (int j = 0; j <= Ls / 2; j++) {
                        const double a = 2.0 * M_PI * j * *shift / Ls;
                        shift_factors[j] = std::complex<T>((T)std::cos(a), (T)std::sin(a));
                    }
                }
                const auto& derfact = shift ? shift_factors
                                    : (ct == PRESSURE) ? disc.pressure_deriv_factors : disc.velocity_deriv_factors;
                RhoArray<T> rho = get_rho_array<T>(d1->rho, self->rho, d2->rho);
                auto field_of = [&](Domain<T>* d) -> Field2<T>& {
                    if (ct == PRESSURE) return d->p0;
                    return (cd == CX) ? d->vx0 : d->vy0;
                };
                Field2<T>& main = field_of(self);
                int nstrips = range_end - range_start;
                auto extract = [&](Domain<T>* d, bool zero) -> Strips<T> {
                    Field2<T>& f = field_of(d);
                    int off = (cd == CX) ? d->top_left.y : d->top_left.x;
                    int first = range_start - off;
                    if (cd == CX) {
                        int len = f.cols;
                        Strips<T> s_(nstrips, len);
                        if (zero) return s_;
                        if (first < 0 || first + nstrips > f.rows)
                            throw OracleError(PSTD_ERR_UNSUPPORTED, "clipped range outside a neighbour (reference reads out of bounds)");
                        for (int r = 0; r < nstrips; r++)
                            for (int c = 0; c < len; c++) s_(r, c) = f(first + r, c);
                        return s_;
                    } else {
                        int len = f.rows;
                        Strips<T> s_(nstrips, len);
                        if (zero) return s_;
                        if (first < 0 || first + nstrips > f.cols)
                            throw OracleError(PSTD_ERR_UNSUPPORTED, "clipped range outside a neighbour (reference reads out of bounds)");
                        for (int c = 0; c < nstrips; c++)
                            for (int r = 0; r < len; r++) s_(c, r) = f(r, first + c);
                        return s_;
                    }
                };
                (void)main;
                Strips<T> m2 = extract(self, false);
                Strips<T> m1 = extract(d1, side1_zero);
                Strips<T> m3 = extract(d2, side2_zero);
                int L = next_2_power((double)(m2.n + 2 * wlen));
                if (L != (int)derfact.size())
                    throw OracleError(PSTD_ERR_UNSUPPORTED,
                                      "transform length differs from derivative-factor length (N+2W is a power of two)");
                Strips<T> res = spatderp3<T>(m1, m2, m3, derfact, rho, wind, wlen, ct);
                int moff = (cd == CX) ? self->top_left.y : self->top_left.x;
                if (cd == CX) {
                    for (int r = 0; r < nstrips; r++)
                        for (int c = 0; c < res.n; c++) source(range_start - moff + r, c) = res(r, c);
                } else {
                    for (int c = 0; c < nstrips; c++)
                        for (int r = 0; r < res.n; r++) source(r, range_start - moff + c) = res(c, r);
                }
            }
        }
    }

    // kernel/Solver.cpp:162-182
    void update_field_values(Domain<T>* d, int rk_step) {
        T dt = (T)s.time_step();
        T c1sq = (T)s.c1 * (T)s.c1;
        T coef = dt * (T)s.rk[rk_step];
        T rho = d->rho;
        for (size_t i = 0; i < d->vx0.a.size(); i++) d->vx0.a[i] = d->pvx0.a[i] - coef * (d->Lpx.a[i] / rho);
        for (size_t i = 0; i < d->vy0.a.size(); i++) d->vy0.a[i] = d->pvy0.a[i] - coef * (d->Lpy.a[i] / rho);
        for (size_t i = 0; i < d->px0.a.size(); i++) d->px0.a[i] = d->ppx0.a[i] - coef * (d->Lvx.a[i] * rho * c1sq);
        for (size_t i = 0; i < d->py0.a.size(); i++) d->py0.a[i] = d->ppy0.a[i] - coef * (d->Lvy.a[i] * rho * c1sq);
    }

    // kernel/Solver.cpp:95-151 ; threads > 1 runs the calc tasks concurrently
    void compute_rk_step(int rk_step, int threads) {
        struct Task { Domain<T>* d; CalcDirection cd; CalcType ct; };
        std::vector<Task> tasks;
        for (int cdi = 0; cdi < 2; cdi++)
            for (int cti = 0; cti < 2; cti++)
                for (auto* d : domain_list)
                    if (!d->rigid && d->should_update[cdi]) tasks.push_back({d, (CalcDirection)cdi, (CalcType)cti});
        if (threads > 1) {
            std::string err; int code = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
            for (int t = 0; t < (int)tasks.size(); t++) {
                try { calc(tasks[t].d, tasks[t].cd, tasks[t].ct); }
                catch (OracleError& e) {
#pragma omp critical
                    { err = e.what(); code = e.code; }
                }
            }
            if (code) throw OracleError(code, err);
        } else {
            for (auto& t : tasks) calc(t.d, t.cd, t.ct);
        }
        for (auto* d : domain_list) if (!d->rigid) update_field_values(d, rk_step);
        for (auto* d : domain_list)
            for (size_t i = 0; i < d->p0.a.size(); i++) d->p0.a[i] = d->px0.a[i] + d->py0.a[i];
    }

    // kernel/Solver.cpp:71-93
    template <class FrameFn>
    void compute_timestep(int frame, int threads, std::vector<double>& rec_out, FrameFn&& on_frame) {
        for (auto* d : domain_list) {
            d->pp0 = d->p0; d->ppx0 = d->px0; d->ppy0 = d->py0; d->pvx0 = d->vx0; d->pvy0 = d->vy0;
        }
        for (int rk = 0; rk < 6; rk++) compute_rk_step(rk, threads);
        for (auto* d : domain_list)
            if (frame % s.save_nth == 0 && !d->is_pml) on_frame(frame, d);
        for (auto* d : domain_list) {
            if (!d->is_pml) continue;
            for (size_t i = 0; i < d->px0.a.size(); i++) d->px0.a[i] *= d->pml_px.a[i];
            for (size_t i = 0; i < d->py0.a.size(); i++) d->py0.a[i] *= d->pml_py.a[i];
            for (size_t i = 0; i < d->vx0.a.size(); i++) d->vx0.a[i] *= d->pml_vx.a[i];
            for (size_t i = 0; i < d->vy0.a.size(); i++) d->vy0.a[i] *= d->pml_vy.a[i];
        }
        for (auto& r : receivers) {
            int rx = r.grid.x - r.container->top_left.x, ry = r.grid.y - r.container->top_left.y;
            rec_out.push_back(spectral ? (double)spectral_sample(r) : (double)r.container->p0(rx, ry));
        }
    }

    // Spectral receiver (own definition; the reference's compute_with_si,
    // kernel/core/Receiver.cpp:85-121, is disabled at :48 and shifts by the
    // integer grid location, :41): p0 of the container D and of its low and
    // high y neighbours shifted along x by gx - ix (calc with shift factors,
    // as calc_domain_fields, :117-121), then D's y strips of that shifted
    // field shifted along y by gy - iy; the value at cell (ix, iy).
    T spectral_sample(const Receiver<T>& r) {
        Domain<T>* D = r.container;
        const double fx = (double)r.gx - r.grid.x, fy = (double)r.gy - r.grid.y;
        std::vector<Domain<T>*> near{D};
        for (auto* e : D->bottom) near.push_back(e);
        for (auto* e : D->top) near.push_back(e);
        std::vector<Field2<T>> shifted;
        for (auto* e : near) {
            Field2<T> f, g;
            f.zeros(e->size.y, e->size.x + 1);
            calc(e, CX, PRESSURE, &fx, &f);
            g.zeros(e->size.y, e->size.x);
            for (int i = 0; i < e->size.y; i++)
                for (int j = 0; j < e->size.x; j++) g(i, j) = f(i, j);
            shifted.push_back(std::move(g));
        }
        for (size_t i = 0; i < near.size(); i++) std::swap(near[i]->p0, shifted[i]);
        Field2<T> out;
        out.zeros(D->size.y + 1, D->size.x);
        try {
            calc(D, CY, PRESSURE, &fy, &out);
        } catch (...) {
            for (size_t i = 0; i < near.size(); i++) std::swap(near[i]->p0, shifted[i]);
            throw;
        }
        for (size_t i = 0; i < near.size(); i++) std::swap(near[i]->p0, shifted[i]);
        return out(r.grid.y - D->top_left.y, r.grid.x - D->top_left.x);
    }
};

// ---------------------------------------------------------------- handle
struct Handle {
    int precision = 32;
    std::unique_ptr<Scene<float>> sf;
    std::unique_ptr<Scene<double>> sd;
    std::vector<double> receivers;   // step-major
    int steps_done = 0;
};

}  // namespace orc

using namespace orc;

typedef void (*orc_frame_cb)(void* user, int32_t frame, int32_t domain, const double* data, int64_t n);

template <class T>
static Scene<T>* scene_of(Handle* h);
template <>
Scene<float>* scene_of<float>(Handle* h) { return h->sf.get(); }
template <>
Scene<double>* scene_of<double>(Handle* h) { return h->sd.get(); }

template <class T, class F>
static int dispatch(Handle* h, F&& f) {
    try { return f(scene_of<T>(h)); }
    catch (OracleError& e) { g_err = e.what(); return e.code; }
    catch (std::exception& e) { g_err = e.what(); return PSTD_ERR_INVALID; }
}

#define ORC_BOTH(h, body) \
    ((h)->precision == 64 ? dispatch<double>((h), [&](auto* sc) body) : dispatch<float>((h), [&](auto* sc) body))

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

int orc_create(const pstd_config* cfg, int32_t precision, Handle** out) {
    *out = nullptr;
    auto h = std::make_unique<Handle>();
    h->precision = precision == 64 ? 64 : 32;
    try {
        if (h->precision == 64) { h->sd = std::make_unique<Scene<double>>(); h->sd->build(cfg); }
        else { h->sf = std::make_unique<Scene<float>>(); h->sf->build(cfg); }
    } catch (OracleError& e) { g_err = e.what(); return e.code; }
    catch (std::exception& e) { g_err = e.what(); return PSTD_ERR_INVALID; }
    *out = h.release();
    return 0;
}

void orc_destroy(Handle* h) { delete h; }

int orc_framecount(Handle* h, int32_t* n) {
    return ORC_BOTH(h, { *n = sc->framecount; return 0; });
}

// Run n_steps time steps (n_steps < 0: framecount).  threads > 1 runs the
// derivative tasks of each RK stage concurrently (MultiThreadSolver).
int orc_run(Handle* h, int32_t n_steps, int32_t threads, orc_frame_cb cb, void* user) {
    return ORC_BOTH(h, {
        int steps = n_steps < 0 ? sc->framecount : n_steps;
        std::vector<double> buf;
        for (int f = 0; f < steps; f++) {
            int frame = h->steps_done;
            sc->compute_timestep(frame, threads, h->receivers, [&](int fr, auto* d) {
                if (!cb) return;
                buf.resize(d->p0.a.size());
                for (size_t i = 0; i < buf.size(); i++) buf[i] = (double)d->p0.a[i];
                cb(user, fr, d->id, buf.data(), (int64_t)buf.size());
            });
            h->steps_done++;
        }
        return 0;
    });
}

int orc_receiver_count(Handle* h, int32_t* n) {
    return ORC_BOTH(h, { *n = (int32_t)sc->receivers.size(); return 0; });
}

int orc_get_receivers(Handle* h, double* dst, int64_t n) {
    if ((size_t)n != h->receivers.size()) { g_err = "size mismatch"; return PSTD_ERR_INVALID; }
    std::memcpy(dst, h->receivers.data(), sizeof(double) * h->receivers.size());
    return 0;
}

int orc_domain_count(Handle* h, int32_t* n) {
    return ORC_BOTH(h, { *n = (int32_t)sc->domain_list.size(); return 0; });
}

int orc_domain_info(Handle* h, int32_t index, pstd_domain_info* o) {
    return ORC_BOTH(h, {
        if (index < 0 || index >= (int)sc->domain_list.size()) { g_err = "bad index"; return PSTD_ERR_INVALID; }
        auto* d = sc->domain_list[index];
        std::memset(o, 0, sizeof *o);
        o->id = d->id;
        o->top_left[0] = d->top_left.x; o->top_left[1] = d->top_left.y;
        o->size[0] = d->size.x; o->size[1] = d->size.y;
        o->is_pml = d->is_pml; o->is_secondary_pml = d->is_secondary_pml; o->is_rigid = d->rigid; o->local = d->local;
        o->should_update[0] = d->should_update[0]; o->should_update[1] = d->should_update[1];
        o->n_neighbours[0] = (int)d->left.size(); o->n_neighbours[1] = (int)d->right.size();
        o->n_neighbours[2] = (int)d->top.size(); o->n_neighbours[3] = (int)d->bottom.size();
        int W = sc->s.window();
        for (int cd = 0; cd < 2; cd++) {
            int n = cd == 0 ? d->size.x : d->size.y;
            int w = W; while (w > n) w /= 2;
            o->window[cd] = w;
            o->fft_length[cd] = (!d->rigid && d->should_update[cd]) ? next_2_power((double)(n + 2 * w)) : 0;
        }
        o->alpha = d->alpha; o->impedance = (float)d->impedance; o->rho = (float)d->rho;
        return 0;
    });
}

int orc_neighbours(Handle* h, int32_t index, int32_t dir, int32_t* out, int32_t cap, int32_t* n) {
    return ORC_BOTH(h, {
        auto* d = sc->domain_list.at(index);
        auto& v = d->nb((Direction)dir);
        *n = (int32_t)v.size();
        for (int i = 0; i < (int)v.size() && i < cap; i++) {
            auto it = std::find(sc->domain_list.begin(), sc->domain_list.end(), v[i]);
            out[i] = (int32_t)(it - sc->domain_list.begin());
        }
        return 0;
    });
}

// field: 0 p0 1 px 2 py 3 vx 4 vy 5..8 pml px py vx vy
int orc_snapshot(Handle* h, int32_t index, int32_t field, double* dst, int64_t n) {
    return ORC_BOTH(h, {
        auto* d = sc->domain_list.at(index);
        auto* f = &d->p0;
        switch (field) {
            case 0: f = &d->p0; break; case 1: f = &d->px0; break; case 2: f = &d->py0; break;
            case 3: f = &d->vx0; break; case 4: f = &d->vy0; break;
            case 5: f = &d->pml_px; break; case 6: f = &d->pml_py; break;
            case 7: f = &d->pml_vx; break; case 8: f = &d->pml_vy; break;
            default: g_err = "bad field"; return PSTD_ERR_INVALID;
        }
        if ((size_t)n != f->a.size()) { g_err = "size mismatch"; return PSTD_ERR_INVALID; }
        for (int64_t i = 0; i < n; i++) dst[i] = (double)f->a[i];
        return 0;
    });
}

// ---- known-answer helpers (reference test/Kernel/*.cpp) ----
int32_t orc_next_2_power(double n) { return next_2_power(n); }
int32_t orc_window_size(float patcherror) { return window_size(patcherror); }

int orc_window(int32_t W, int32_t patch_error, int32_t precision, double* out) {
    if (precision == 64) { auto w = window_coefficients<double>(W, patch_error); std::copy(w.begin(), w.end(), out); }
    else { auto w = window_coefficients<float>(W, patch_error); for (size_t i = 0; i < w.size(); i++) out[i] = w[i]; }
    return 0;
}

int orc_rho_array(double rho1, double rho_self, double rho2, int32_t precision, double* out16) {
    if (precision == 64) {
        auto r = get_rho_array<double>(rho1, rho_self, rho2);
        for (int i = 0; i < 8; i++) { out16[i] = r.pressure[i / 2][i % 2]; out16[8 + i] = r.velocity[i / 2][i % 2]; }
    } else {
        auto r = get_rho_array<float>((float)rho1, (float)rho_self, (float)rho2);
        for (int i = 0; i < 8; i++) { out16[i] = r.pressure[i / 2][i % 2]; out16[8 + i] = r.velocity[i / 2][i % 2]; }
    }
    return 0;
}

// wave numbers, complex factor imag parts, pressure and velocity factors (re, im interleaved)
int orc_discretization(float dx, int32_t N, int32_t precision, int32_t* len, double* k, double* cimag,
                       double* pd, double* vd, int32_t cap) {
    auto fill = [&](auto d) {
        int n = (int)d.wave_numbers.size();
        *len = n;
        for (int i = 0; i < n && i < cap; i++) {
            k[i] = d.wave_numbers[i]; cimag[i] = d.complex_factors[i].imag();
            pd[2 * i] = d.pressure_deriv_factors[i].real(); pd[2 * i + 1] = d.pressure_deriv_factors[i].imag();
            vd[2 * i] = d.velocity_deriv_factors[i].real(); vd[2 * i + 1] = d.velocity_deriv_factors[i].imag();
        }
    };
    if (precision == 64) fill(discretize_wave_numbers<double>((double)dx, match_number(N)));
    else fill(discretize_wave_numbers<float>(dx, match_number(N)));
    return 0;
}

// spatderp3 on single strips (X direction, batch 1) with the given derfact
int orc_spatderp3(const double* p1, int32_t n1, const double* p2, int32_t n2, const double* p3, int32_t n3,
                  const double* derfact_reim, int32_t dlen, const double* window, int32_t wlen,
                  double rho1, double rho_self, double rho2, int32_t velocity, int32_t precision, double* out) {
    auto run = [&](auto tag) -> int {
        using T = decltype(tag);
        Strips<T> a(1, n1), b(1, n2), c(1, n3);
        for (int i = 0; i < n1; i++) a(0, i) = (T)p1[i];
        for (int i = 0; i < n2; i++) b(0, i) = (T)p2[i];
        for (int i = 0; i < n3; i++) c(0, i) = (T)p3[i];
        std::vector<std::complex<T>> df(dlen);
        for (int i = 0; i < dlen; i++) df[i] = std::complex<T>((T)derfact_reim[2 * i], (T)derfact_reim[2 * i + 1]);
        std::vector<T> w(2 * wlen + 1);
        for (int i = 0; i < 2 * wlen + 1; i++) w[i] = (T)window[i];
        auto rho = get_rho_array<T>((T)rho1, (T)rho_self, (T)rho2);
        auto r = spatderp3<T>(a, b, c, df, rho, w, wlen, velocity ? VELOCITY : PRESSURE);
        for (int i = 0; i < r.n; i++) out[i] = (double)r(0, i);
        return 0;
    };
    try { return precision == 64 ? run(0.0) : run(0.0f); }
    catch (OracleError& e) { g_err = e.what(); return e.code; }
}

// Speed of the oracle's own strip transform (float): n_strips strips of
// length L through r2c, a complex multiply per bin and c2r -- the transform
// core of spatderp3 -- on `threads` OpenMP threads, best of `reps` runs.  Lets
// a caller set the oracle's FFT beside another FFT library on the same shapes,
// so the oracle's speed is not read as FFTW's.
int32_t orc_fft_seconds(int32_t L, int32_t n_strips, int32_t threads, int32_t reps, double* seconds) {
    if (L < 4 || (L & (L - 1)) || n_strips < 1 || threads < 1 || reps < 1 || !seconds) {
        g_err = "orc_fft_seconds: bad arguments";
        return PSTD_ERR_INVALID;
    }
    std::vector<float> data((size_t)n_strips * L);
    for (size_t i = 0; i < data.size(); i++) data[i] = (float)((i * 2654435761u) % 1000) * 1e-3f;
    std::vector<std::complex<float>> filt(L / 2 + 1, std::complex<float>(0.5f, 0.25f));
    double best = 1e30;
    for (int r = 0; r < reps; r++) {
        const double t0 = omp_get_wtime();
#pragma omp parallel num_threads(threads)
        {
            const RealFFT<float>& plan = fft_plan<float>(L);
            std::vector<std::complex<float>> spec(L / 2 + 1), work(L / 2 + 1);
#pragma omp for schedule(static)
            for (int s = 0; s < n_strips; s++) {
                float* x = data.data() + (size_t)s * L;
                plan.r2c(x, spec.data(), work.data());
                for (int k = 0; k <= L / 2; k++) spec[k] *= filt[k];
                plan.c2r(spec.data(), x, work.data());
            }
        }
        best = std::min(best, omp_get_wtime() - t0);
    }
    *seconds = best;
    return 0;
}

int32_t orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
