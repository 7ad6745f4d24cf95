// stage_kernel.cuh -- one RK stage of the strip-derivative solve, sm_103a.
//
// A CTA takes one job: up to 2*CS adjacent strips (rows for x, columns for
// y) of one domain sharing both interface neighbours, and computes for each
// the reference's windowed Fourier derivative (kernel/core/kernel_functions.cpp:
// 123-318) fused with the RK stage update (kernel/Solver.cpp:162-182):
//
//   1. gather: strip + the two W-wide interface bands of the neighbours
//      (reflected / transmitted and windowed, kernel/core/kernel_functions.cpp:
//      191-216,246-269), zero padded to L, two real strips per complex strip,
//      in shared memory; p0 is formed as px + py of the previous stage while
//      loading;
//   2. forward complex FFT of length L in place (decimation in frequency,
//      radix 16/8/4/2 butterflies in registers, twiddles from an FP64-built
//      table), output in digit-reversed position order;
//   3. multiply by the Hermitian-extended derivative filter i k e^{-/+ i k dx/2}
//      (1/L folded in) stored in the same position order, fused with the last
//      forward and the first inverse pass;
//   4. inverse FFT (decimation in time), natural order;
//   5. epilogue: slice W..W+n and RK-update against the stage-start set
//      (vx/vy get the PML multiply of the sixth stage here).
//
// Packing two real strips into one complex strip is exact in real
// arithmetic: the filter is Hermitian, so the operator is real and acts on
// the real and imaginary parts separately.
#pragma once
#include <cuda_runtime.h>

#include "launch.hpp"

namespace pstd {

// ---------------------------------------------------------------- complex helpers
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {   // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <bool INV>
__device__ __forceinline__ float2 rot(float2 a) {   // * -i (forward) or * +i (inverse)
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// cos / sin of multiples of pi/8
#define PSTD_C8 0.92387953251128674f
#define PSTD_S8 0.38268343236508978f
#define PSTD_R2 0.70710678118654752f

template <int K, bool INV>
__device__ __forceinline__ float2 tw16(float2 a) {   // a * exp(-/+ 2 pi i K / 16)
    constexpr float sg = INV ? 1.f : -1.f;
    if (K == 0) return a;
    if (K == 4) return rot<INV>(a);
    if (K == 2) return cmul(a, make_float2(PSTD_R2, sg * PSTD_R2));
    if (K == 6) return cmul(a, make_float2(-PSTD_R2, sg * PSTD_R2));
    if (K == 1) return cmul(a, make_float2(PSTD_C8, sg * PSTD_S8));
    if (K == 3) return cmul(a, make_float2(PSTD_S8, sg * PSTD_C8));
    if (K == 5) return cmul(a, make_float2(-PSTD_S8, sg * PSTD_C8));
    return cmul(a, make_float2(-PSTD_C8, sg * PSTD_S8));
}

template <int R, bool INV>
struct DFT;
template <bool INV>
struct DFT<2, INV> {
    static __device__ __forceinline__ void run(float2* x) {
        float2 a = x[0], b = x[1];
        x[0] = cadd(a, b);
        x[1] = csub(a, b);
    }
};
template <bool INV>
struct DFT<4, INV> {
    static __device__ __forceinline__ void run(float2* x) {
        float2 a = cadd(x[0], x[2]), b = csub(x[0], x[2]);
        float2 c = cadd(x[1], x[3]), d = rot<INV>(csub(x[1], x[3]));
        x[0] = cadd(a, c);
        x[2] = csub(a, c);
        x[1] = cadd(b, d);
        x[3] = csub(b, d);
    }
};
template <bool INV>
struct DFT<8, INV> {
    static __device__ __forceinline__ void run(float2* x) {
        float2 e[4] = {x[0], x[2], x[4], x[6]};
        float2 o[4] = {x[1], x[3], x[5], x[7]};
        DFT<4, INV>::run(e);
        DFT<4, INV>::run(o);
        o[1] = tw16<2, INV>(o[1]);
        o[2] = tw16<4, INV>(o[2]);
        o[3] = tw16<6, INV>(o[3]);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            x[k] = cadd(e[k], o[k]);
            x[k + 4] = csub(e[k], o[k]);
        }
    }
};
template <bool INV>
struct DFT<16, INV> {
    static __device__ __forceinline__ void run(float2* x) {
        float2 e[8], o[8];
#pragma unroll
        for (int k = 0; k < 8; k++) { e[k] = x[2 * k]; o[k] = x[2 * k + 1]; }
        DFT<8, INV>::run(e);
        DFT<8, INV>::run(o);
        o[1] = tw16<1, INV>(o[1]);
        o[2] = tw16<2, INV>(o[2]);
        o[3] = tw16<3, INV>(o[3]);
        o[4] = tw16<4, INV>(o[4]);
        o[5] = tw16<5, INV>(o[5]);
        o[6] = tw16<6, INV>(o[6]);
        o[7] = tw16<7, INV>(o[7]);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            x[k] = cadd(e[k], o[k]);
            x[k + 8] = csub(e[k], o[k]);
        }
    }
};

// ---------------------------------------------------------------- variant
template <int L_, int CS_, int NT_, int MINB_, int R0_, int R1_, int R2_ = 0, int R3_ = 0>
struct Cfg {
    static constexpr int L = L_, CS = CS_, NT = NT_, MINB = MINB_;
    static constexpr int R0 = R0_, R1 = R1_, R2 = R2_, R3 = R3_;
    static constexpr int NP = R3_ ? 4 : (R2_ ? 3 : 2);
    static_assert(R0 * R1 * (R2 ? R2 : 1) * (R3 ? R3 : 1) == L, "radix plan must multiply to L");
    // strip pitch in float2: L + 16/CS (mod 16), so that the CS strips a
    // half-warp touches at one offset fall in distinct bank pairs
    static constexpr int PAD = CS >= 16 ? 1 : 16 / CS;
    static constexpr int SP = L + PAD;
    static constexpr int SMEM = CS * SP * 8;
};

// Twiddles of a pass with block size M and radix R live in a table
// [n1][k] = exp(-2 pi i n1 k / M), n1 < M/R, k < R (k = 0 included so a row
// is R float2 = R/2 aligned 16-byte loads); TOFF is the pass' offset.
template <int R>
__device__ __forceinline__ void load_twiddles(const float2* __restrict__ row, float2 (&w)[R]) {
    const float4* t4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int h = 0; h < R / 2; h++) {
        const float4 v = __ldg(t4 + h);
        w[2 * h] = make_float2(v.x, v.y);
        w[2 * h + 1] = make_float2(v.z, v.w);
    }
}

template <class C, int R, int M, int TOFF>
__device__ __forceinline__ void fwd_pass(float2* sm, const float2* __restrict__ tw) {
    constexpr int Q = M / R;
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it = threadIdx.x; it < ITEMS; it += C::NT) {
        const int cs = it % C::CS, b = it / C::CS;
        const int blk = b / Q, n1 = b % Q;
        float2 w[R];
        if (Q > 1) load_twiddles<R>(tw + TOFF + n1 * R, w);
        float2* base = sm + cs * C::SP + blk * M + n1;
        float2 x[R];
#pragma unroll
        for (int q = 0; q < R; q++) x[q] = base[q * Q];
        DFT<R, false>::run(x);
        if (Q > 1) {
#pragma unroll
            for (int k = 1; k < R; k++) x[k] = cmul(x[k], w[k]);
        }
#pragma unroll
        for (int k = 0; k < R; k++) base[k * Q] = x[k];
    }
}

template <class C, int R, int M, int TOFF>
__device__ __forceinline__ void inv_pass(float2* sm, const float2* __restrict__ tw) {
    constexpr int Q = M / R;
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it = threadIdx.x; it < ITEMS; it += C::NT) {
        const int cs = it % C::CS, b = it / C::CS;
        const int blk = b / Q, n1 = b % Q;
        float2 w[R];
        if (Q > 1) load_twiddles<R>(tw + TOFF + n1 * R, w);
        float2* base = sm + cs * C::SP + blk * M + n1;
        float2 x[R];
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = base[k * Q];
        if (Q > 1) {
#pragma unroll
            for (int k = 1; k < R; k++) x[k] = cmulc(x[k], w[k]);
        }
        DFT<R, true>::run(x);
#pragma unroll
        for (int q = 0; q < R; q++) base[q * Q] = x[q];
    }
}

template <class C, int R>
__device__ __forceinline__ void mid_pass(float2* sm, const float2* __restrict__ filt) {
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it = threadIdx.x; it < ITEMS; it += C::NT) {
        const int cs = it % C::CS, blk = it / C::CS;
        float2* base = sm + cs * C::SP + blk * R;
        float2 x[R];
#pragma unroll
        for (int q = 0; q < R; q++) x[q] = base[q];
        DFT<R, false>::run(x);
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = cmul(x[k], __ldg(&filt[blk * R + k]));
        DFT<R, true>::run(x);
#pragma unroll
        for (int q = 0; q < R; q++) base[q] = x[q];
    }
}

template <class C>
__device__ __forceinline__ void convolve(float2* sm, const float2* __restrict__ tw, const float2* __restrict__ filt) {
    constexpr int M0 = C::L, M1 = M0 / C::R0;
    constexpr int T0 = 0, T1 = M0;   // pass table offsets (a pass' table holds M entries)
    if constexpr (C::NP == 2) {
        fwd_pass<C, C::R0, M0, T0>(sm, tw);
        __syncthreads();
        mid_pass<C, C::R1>(sm, filt);
        __syncthreads();
        inv_pass<C, C::R0, M0, T0>(sm, tw);
    } else if constexpr (C::NP == 3) {
        fwd_pass<C, C::R0, M0, T0>(sm, tw);
        __syncthreads();
        fwd_pass<C, C::R1, M1, T1>(sm, tw);
        __syncthreads();
        mid_pass<C, C::R2>(sm, filt);
        __syncthreads();
        inv_pass<C, C::R1, M1, T1>(sm, tw);
        __syncthreads();
        inv_pass<C, C::R0, M0, T0>(sm, tw);
    } else {
        constexpr int M2 = M1 / C::R1, T2 = M0 + M1;
        fwd_pass<C, C::R0, M0, T0>(sm, tw);
        __syncthreads();
        fwd_pass<C, C::R1, M1, T1>(sm, tw);
        __syncthreads();
        fwd_pass<C, C::R2, M2, T2>(sm, tw);
        __syncthreads();
        mid_pass<C, C::R3>(sm, filt);
        __syncthreads();
        inv_pass<C, C::R2, M2, T2>(sm, tw);
        __syncthreads();
        inv_pass<C, C::R1, M1, T1>(sm, tw);
        __syncthreads();
        inv_pass<C, C::R0, M0, T0>(sm, tw);
    }
}

// reference operation order: dom = (band * T + mirror * R) * window
__device__ __forceinline__ float band_value(float raw, float mirror, float T, float R, float w) {
    return __fmul_rn(__fadd_rn(__fmul_rn(raw, T), __fmul_rn(mirror, R)), w);
}

// Source of the strip data of one domain in one stage.
struct Src {
    const float* a;   // p0 array (stale) or px, or the velocity field
    const float* b;   // py (p0 formed on the fly) or nullptr
    int pitch;
    __device__ __forceinline__ float at(long long e) const {
        return b ? __fadd_rn(__ldg(a + e), __ldg(b + e)) : __ldg(a + e);
    }
};

__device__ __forceinline__ Src strip_source(const StageArgs& A, const DevDomain& D, bool vel, bool ydir, bool first) {
    const float* base = D.fixed ? A.fixed : A.in;
    Src s;
    if (vel) {
        s.a = base + (ydir ? D.o_vy : D.o_vx);
        s.b = nullptr;
        s.pitch = ydir ? D.pitch_vy : D.pitch_vx;
    } else if (A.stage == 0 && (D.pml || first)) {
        s.a = A.p0 + D.o_p0;   // p0 the reference reads at the first stage (stale / initial)
        s.b = nullptr;
        s.pitch = D.pitch_p;
    } else {
        s.a = base + D.o_px;
        s.b = base + D.o_py;
        s.pitch = D.pitch_p;
    }
    return s;
}

__device__ __forceinline__ float4 ld4(const float* p, int i, int n) {
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i + 4 <= n) {
        u = __ldg(reinterpret_cast<const float4*>(p + i));
    } else {
        u.x = __ldg(p + i);
        if (i + 1 < n) u.y = __ldg(p + i + 1);
        if (i + 2 < n) u.z = __ldg(p + i + 2);
    }
    return u;
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}

// Carry the fields of a non-updated axis through the stage: the derivative
// array keeps its zero content, so the RK update returns the stage-start value.
static __device__ void copy_axis(const StageArgs& A, const DevDomain& D, bool ydir) {
    const int nt = blockDim.x;
    if (!ydir) {
        for (int k = threadIdx.x; k < D.ny * (D.nx + 1); k += nt) {
            const int r = k / (D.nx + 1), i = k - r * (D.nx + 1);
            const long long e = D.o_vx + (long long)r * D.pitch_vx + i;
            float v = A.prev[e];
            if (A.last && D.att_xv >= 0) v = __fmul_rn(v, A.att[D.att_xv + i]);
            A.out[e] = v;
        }
        for (int k = threadIdx.x; k < D.ny * D.nx; k += nt) {
            const int r = k / D.nx, i = k - r * D.nx;
            const long long e = D.o_px + (long long)r * D.pitch_p + i;
            A.out[e] = A.prev[e];
        }
    } else {
        for (int k = threadIdx.x; k < (D.ny + 1) * D.nx; k += nt) {
            const int r = k / D.nx, i = k - r * D.nx;
            const long long e = D.o_vy + (long long)r * D.pitch_vy + i;
            float v = A.prev[e];
            if (A.last && D.att_yv >= 0) v = __fmul_rn(v, A.att[D.att_yv + r]);
            A.out[e] = v;
        }
        for (int k = threadIdx.x; k < D.ny * D.nx; k += nt) {
            const int r = k / D.nx, i = k - r * D.nx;
            const long long e = D.o_py + (long long)r * D.pitch_p + i;
            A.out[e] = A.prev[e];
        }
    }
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_kernel(StageArgs A) {
    constexpr int CS = C::CS, NT = C::NT, SP = C::SP, L = C::L;
    constexpr int S2 = 2 * CS;
    extern __shared__ float2 sm[];
    float* smf = reinterpret_cast<float*>(sm);
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    const bool ydir = job.kind & JK_Y;
    if (job.kind & JK_COPY) {
        copy_axis(A, dom, ydir);
        return;
    }
    const bool vel = job.kind & JK_VEL;
    const bool first = *A.first_step != 0;
    const int W = job.W;
    const int n = (ydir ? dom.ny : dom.nx) + (vel ? 1 : 0);   // strip length
    const int count = job.count;
    const Src S = strip_source(A, dom, vel, ydir, first);

    // ---- 1. gather -------------------------------------------------------
    constexpr int NW = NT / 32;                   // warps
    constexpr int WPP = NW >= CS ? NW / CS : 1;   // warps per strip pair
    constexpr int PST = NW / WPP;                 // strip pairs in flight
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (!ydir) {
        // row pairs (2cs, 2cs+1), 16-byte loads, two chunks per lane in flight
        const int chunks = (n + 3) >> 2;
        for (int cs = warp / WPP; cs < CS; cs += PST) {
            const int s0 = 2 * cs;
            const float* a0 = S.a + (long long)(job.first + s0) * S.pitch;
            const float* b0 = S.b ? S.b + (long long)(job.first + s0) * S.pitch : nullptr;
            const bool h0 = s0 < count, h1 = s0 + 1 < count;
            for (int c0 = (warp % WPP) * 32 + lane; c0 < chunks; c0 += 2 * WPP * 32) {
                float4 u[2], v[2];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int c = c0 + q * WPP * 32, i = c << 2;
                    u[q] = v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (c < chunks) {
                        if (h0) u[q] = b0 ? add4(ld4(a0, i, n), ld4(b0, i, n)) : ld4(a0, i, n);
                        if (h1) v[q] = b0 ? add4(ld4(a0 + S.pitch, i, n), ld4(b0 + S.pitch, i, n)) : ld4(a0 + S.pitch, i, n);
                    }
                }
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int c = c0 + q * WPP * 32, i = c << 2;
                    if (c < chunks) {
                        float2* d = sm + cs * SP + W + i;
                        d[0] = make_float2(u[q].x, v[q].x);
                        if (i + 1 < n) d[1] = make_float2(u[q].y, v[q].y);
                        if (i + 2 < n) d[2] = make_float2(u[q].z, v[q].z);
                        if (i + 3 < n) d[3] = make_float2(u[q].w, v[q].w);
                    }
                }
            }
        }
    } else {
        // columns: consecutive threads read consecutive columns of one row,
        // four elements per thread in flight
        const int total = S2 * n;
        for (int f0 = threadIdx.x; f0 < total; f0 += 4 * NT) {
            float val[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NT;
                val[q] = 0.f;
                if (f < total) {
                    const int s = f % S2, i = f / S2;
                    if (s < count) val[q] = S.at((long long)i * S.pitch + job.first + s);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NT;
                if (f < total) {
                    const int s = f % S2, i = f / S2;
                    smf[2 * ((s >> 1) * SP + W + i) + (s & 1)] = val[q];
                }
            }
        }
    }
    // interface bands and zero padding
    {
        const float* wl = A.win + job.wtab;          // window.head(W)
        const float* wr = A.win + job.wtab + W + 1;  // window.tail(W)
        Src S1{nullptr, nullptr, 0}, S3{nullptr, nullptr, 0};
        int n1 = 0;
        if (job.d1 >= 0) {
            const DevDomain D1 = A.doms[job.d1];
            S1 = strip_source(A, D1, vel, ydir, first);
            n1 = (ydir ? D1.ny : D1.nx) + (vel ? 1 : 0);
        }
        if (job.d2 >= 0) S3 = strip_source(A, A.doms[job.d2], vel, ydir, first);
        // bands: one warp per strip, lanes along the band
        for (int s = warp; s < S2; s += NW) {
            const bool live = s < count;
            for (int j = lane; j < 2 * W; j += 32) {
                float val = 0.f;
                int pos;
                if (j < W) {
                    pos = j;
                    if (live && job.d1 >= 0) {
                        const int e1 = vel ? n1 - W - 1 + j : n1 - W + j;   // far end of the low neighbour
                        const int m = vel ? W - j : W - 1 - j;              // mirrored own element
                        float raw, mir;
                        if (!ydir) {
                            raw = S1.at((long long)(job.o1 + s) * S1.pitch + e1);
                            mir = S.at((long long)(job.first + s) * S.pitch + m);
                        } else {
                            raw = S1.at((long long)e1 * S1.pitch + job.o1 + s);
                            mir = S.at((long long)m * S.pitch + job.first + s);
                        }
                        val = band_value(raw, mir, job.T1, job.R1, wl[j]);
                    }
                } else {
                    const int jj = j - W;
                    pos = W + n + jj;
                    if (live && job.d2 >= 0) {
                        const int e2 = vel ? 1 + jj : jj;                   // near end of the high neighbour
                        const int m = vel ? n - 2 - jj : n - 1 - jj;
                        float raw, mir;
                        if (!ydir) {
                            raw = S3.at((long long)(job.o2 + s) * S3.pitch + e2);
                            mir = S.at((long long)(job.first + s) * S.pitch + m);
                        } else {
                            raw = S3.at((long long)e2 * S3.pitch + job.o2 + s);
                            mir = S.at((long long)m * S.pitch + job.first + s);
                        }
                        val = band_value(raw, mir, job.T2, job.R2, wr[jj]);
                    }
                }
                smf[2 * ((s >> 1) * SP + pos) + (s & 1)] = val;
            }
        }
        // zero padding [2W+n, L) of every complex strip
        const int z0 = 2 * W + n;
        for (int cs = warp; cs < CS; cs += NW)
            for (int p = z0 + lane; p < L; p += 32) sm[cs * SP + p] = make_float2(0.f, 0.f);
    }
    __syncthreads();

    // ---- 2-4. FFT, derivative filter, inverse FFT -------------------------
    convolve<C>(sm, A.tw, A.filt + job.dtab);
    __syncthreads();

    // ---- 5. epilogue -------------------------------------------------------
    const float cdt = A.doms[job.dom].cdt[A.stage];
    const float rho = dom.rho;
    const int nout = vel ? n - 1 : n + 1;   // cells (vel) or faces (pressure)
    long long fo;
    int fp, ao;
    if (!vel) { fo = ydir ? dom.o_vy : dom.o_vx; fp = ydir ? dom.pitch_vy : dom.pitch_vx; ao = ydir ? dom.att_yv : dom.att_xv; }
    else { fo = ydir ? dom.o_py : dom.o_px; fp = dom.pitch_p; ao = -1; }
    const bool att = A.last && ao >= 0;
    const float c2 = dom.c2;
    if (!ydir) {
        for (int cs = warp / WPP; cs < CS; cs += PST) {
            const float2* srow = sm + cs * SP + W;
            for (int i = (warp % WPP) * 32 + lane; i < nout; i += WPP * 32) {
                const float2 d = srow[i];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = 2 * cs + h;
                    if (s >= count) break;
                    const float dv = h ? d.y : d.x;
                    const long long e = fo + (long long)(job.first + s) * fp + i;
                    float v;
                    if (!vel) {
                        v = __fsub_rn(A.prev[e], __fmul_rn(cdt, __fdiv_rn(dv, rho)));
                        if (att) v = __fmul_rn(v, A.att[ao + i]);
                    } else {
                        v = __fsub_rn(A.prev[e], __fmul_rn(cdt, __fmul_rn(__fmul_rn(dv, rho), c2)));
                    }
                    A.out[e] = v;
                }
            }
        }
    } else {
        for (int f = threadIdx.x; f < S2 * nout; f += NT) {
            const int s = f % S2, i = f / S2;
            if (s >= count) continue;
            const float dv = smf[2 * ((s >> 1) * SP + W + i) + (s & 1)];
            const long long e = fo + (long long)i * fp + job.first + s;
            float v;
            if (!vel) {
                v = __fsub_rn(A.prev[e], __fmul_rn(cdt, __fdiv_rn(dv, rho)));
                if (att) v = __fmul_rn(v, A.att[ao + i]);
            } else {
                v = __fsub_rn(A.prev[e], __fmul_rn(cdt, __fmul_rn(__fmul_rn(dv, rho), c2)));
            }
            A.out[e] = v;
        }
    }
}

template <class C>
cudaError_t launch_stage_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    stage_kernel<C><<<n_jobs, C::NT, C::SMEM, st>>>(a);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_stage_t() {
    return cudaFuncSetAttribute(stage_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
}

template <class C>
StageVariant make_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT; v.smem = C::SMEM; v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.launch = &launch_stage_t<C>;
    v.prepare = &prepare_stage_t<C>;
    v.name = name;
    return v;
}

}  // namespace pstd
