// kernels.cu -- sm_103a kernels of the PSTD time step.
//
// pass_kernel<L>: one CTA takes up to 2*CS adjacent strips (rows for the
// x pass, columns for the y pass) of one domain and computes, for each, the
// reference's windowed Fourier derivative (kernel/core/kernel_functions.cpp:
// 123-318) fused with the RK stage update (kernel/Solver.cpp:162-182) and, at
// the sixth stage, the PML multiply (kernel/core/Domain.cpp:716-725):
//
//   1. gather: strip + the two W-wide interface bands of the neighbours,
//      reflected/transmitted and windowed, zero padded to L, written as
//      interleaved complex numbers (two real strips per complex strip) into
//      shared memory;
//   2. forward complex FFT of length L, in place, decimation in frequency
//      (radix 16/8/4/2 butterflies in registers, twiddles from an FP64-built
//      table), output in digit-reversed position order;
//   3. multiply by the Hermitian-extended derivative filter (i k e^{-/+ i k dx/2},
//      1/L folded in) stored in the same position order -- fused with the
//      last forward and the first inverse pass so those stay in registers;
//   4. inverse FFT (decimation in time), natural order;
//   5. epilogue: slice W..W+n, RK update against the stage-start set, PML.
//
// Packing two real strips as one complex strip is exact in real arithmetic:
// the filter is Hermitian, so the operator is real and acts on the real and
// imaginary parts separately.
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
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// exp(-/+ 2 pi i k / 16) constants (cos and sin of multiples of pi/8)
#define PSTD_C8 0.92387953251128674f
#define PSTD_S8 0.38268343236508978f
#define PSTD_R2 0.70710678118654752f

template <int K, bool INV>
__device__ __forceinline__ float2 tw16(float2 a) {
    // a * exp(-/+ 2 pi i K / 16)
    constexpr float sg = INV ? 1.f : -1.f;
    if (K == 0) return a;
    if (K == 4) return rot<INV>(a);
    if (K == 2) return cmul(a, make_float2(PSTD_R2, sg * PSTD_R2));
    if (K == 6) return cmul(a, make_float2(-PSTD_R2, sg * PSTD_R2));
    if (K == 1) return cmul(a, make_float2(PSTD_C8, sg * PSTD_S8));
    if (K == 3) return cmul(a, make_float2(PSTD_S8, sg * PSTD_C8));
    if (K == 5) return cmul(a, make_float2(-PSTD_S8, sg * PSTD_C8));
    return cmul(a, make_float2(-PSTD_C8, sg * PSTD_S8));   // K == 7
}

// in-register DFT of R points, natural order in and out
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

// ---------------------------------------------------------------- launch shapes
// radix plan, complex strips per CTA and threads per CTA for each length L
template <int L>
struct Shape;
template <> struct Shape<32>   { static constexpr int CS = 16, NT = 64,  NP = 2, R0 = 8,  R1 = 4,  R2 = 0,  R3 = 0; };
template <> struct Shape<64>   { static constexpr int CS = 16, NT = 128, NP = 2, R0 = 8,  R1 = 8,  R2 = 0,  R3 = 0; };
template <> struct Shape<128>  { static constexpr int CS = 16, NT = 128, NP = 2, R0 = 16, R1 = 8,  R2 = 0,  R3 = 0; };
template <> struct Shape<256>  { static constexpr int CS = 16, NT = 256, NP = 2, R0 = 16, R1 = 16, R2 = 0,  R3 = 0; };
template <> struct Shape<512>  { static constexpr int CS = 8,  NT = 256, NP = 3, R0 = 8,  R1 = 8,  R2 = 8,  R3 = 0; };
template <> struct Shape<1024> { static constexpr int CS = 8,  NT = 256, NP = 3, R0 = 16, R1 = 8,  R2 = 8,  R3 = 0; };
template <> struct Shape<2048> { static constexpr int CS = 8,  NT = 512, NP = 3, R0 = 16, R1 = 16, R2 = 8,  R3 = 0; };
template <> struct Shape<4096> { static constexpr int CS = 4,  NT = 512, NP = 3, R0 = 16, R1 = 16, R2 = 16, R3 = 0; };
template <> struct Shape<8192> { static constexpr int CS = 2,  NT = 512, NP = 4, R0 = 16, R1 = 16, R2 = 8,  R3 = 4; };

template <int L>
struct Geo {
    static constexpr int CS = Shape<L>::CS;
    static constexpr int NT = Shape<L>::NT;
    // strip pitch in float2: L + pad with pad = 16/CS (mod 16) so that a
    // half-warp touching the same offset of 16/pad-spaced strips is conflict free
    static constexpr int PAD = CS >= 16 ? 1 : 16 / CS;
    static constexpr int SP = L + PAD;
    static constexpr int SMEM = CS * SP * 8;
};

template <int L, int R, int M>
__device__ __forceinline__ void fwd_pass(float2* sm, const float2* __restrict__ tw) {
    constexpr int CS = Geo<L>::CS, NT = Geo<L>::NT, SP = Geo<L>::SP;
    constexpr int Q = M / R;
    constexpr int ITEMS = CS * (L / R);
    for (int it = threadIdx.x; it < ITEMS; it += NT) {
        const int cs = it % CS, b = it / CS;
        const int blk = b / Q, n1 = b % Q;
        float2* base = sm + cs * SP + blk * M + n1;
        float2 x[R];
#pragma unroll
        for (int q = 0; q < R; q++) x[q] = base[q * Q];
        DFT<R, false>::run(x);
        if (Q > 1) {
#pragma unroll
            for (int k = 1; k < R; k++) x[k] = cmul(x[k], __ldg(&tw[(L / M) * n1 * k]));
        }
#pragma unroll
        for (int k = 0; k < R; k++) base[k * Q] = x[k];
    }
}

template <int L, int R, int M>
__device__ __forceinline__ void inv_pass(float2* sm, const float2* __restrict__ tw) {
    constexpr int CS = Geo<L>::CS, NT = Geo<L>::NT, SP = Geo<L>::SP;
    constexpr int Q = M / R;
    constexpr int ITEMS = CS * (L / R);
    for (int it = threadIdx.x; it < ITEMS; it += NT) {
        const int cs = it % CS, b = it / CS;
        const int blk = b / Q, n1 = b % Q;
        float2* base = sm + cs * SP + blk * M + n1;
        float2 x[R];
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = base[k * Q];
        if (Q > 1) {
#pragma unroll
            for (int k = 1; k < R; k++) x[k] = cmulc(x[k], __ldg(&tw[(L / M) * n1 * k]));
        }
        DFT<R, true>::run(x);
#pragma unroll
        for (int q = 0; q < R; q++) base[q * Q] = x[q];
    }
}

// last forward pass (blocks of R contiguous positions), filter, first inverse pass
template <int L, int R>
__device__ __forceinline__ void mid_pass(float2* sm, const float2* __restrict__ filt) {
    constexpr int CS = Geo<L>::CS, NT = Geo<L>::NT, SP = Geo<L>::SP;
    constexpr int ITEMS = CS * (L / R);
    for (int it = threadIdx.x; it < ITEMS; it += NT) {
        const int cs = it % CS, blk = it / CS;
        float2* base = sm + cs * SP + blk * R;
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

template <int L>
__device__ __forceinline__ void convolve(float2* sm, const float2* __restrict__ tw, const float2* __restrict__ filt) {
    using S = Shape<L>;
    constexpr int M0 = L, M1 = M0 / S::R0, M2 = (S::NP > 1) ? M1 / S::R1 : 1, M3 = (S::NP > 2) ? M2 / S::R2 : 1;
    if constexpr (S::NP == 2) {
        fwd_pass<L, S::R0, M0>(sm, tw);
        __syncthreads();
        mid_pass<L, S::R1>(sm, filt);
        __syncthreads();
        inv_pass<L, S::R0, M0>(sm, tw);
    } else if constexpr (S::NP == 3) {
        fwd_pass<L, S::R0, M0>(sm, tw);
        __syncthreads();
        fwd_pass<L, S::R1, M1>(sm, tw);
        __syncthreads();
        mid_pass<L, S::R2>(sm, filt);
        __syncthreads();
        inv_pass<L, S::R1, M1>(sm, tw);
        __syncthreads();
        inv_pass<L, S::R0, M0>(sm, tw);
    } else {
        fwd_pass<L, S::R0, M0>(sm, tw);
        __syncthreads();
        fwd_pass<L, S::R1, M1>(sm, tw);
        __syncthreads();
        fwd_pass<L, S::R2, M2>(sm, tw);
        __syncthreads();
        mid_pass<L, S::R3>(sm, filt);
        __syncthreads();
        inv_pass<L, S::R2, M2>(sm, tw);
        __syncthreads();
        inv_pass<L, S::R1, M1>(sm, tw);
        __syncthreads();
        inv_pass<L, S::R0, M0>(sm, tw);
    }
    (void)M3;
}

// reference operation order: dom = (band * T + mirror * R) * window
__device__ __forceinline__ float band_value(float raw, float mirror, float T, float R, float w) {
    return __fmul_rn(__fadd_rn(__fmul_rn(raw, T), __fmul_rn(mirror, R)), w);
}

template <int L>
__global__ void __launch_bounds__(Shape<L>::NT, 1) pass_kernel(PassArgs a) {
    constexpr int CS = Geo<L>::CS, NT = Geo<L>::NT, SP = Geo<L>::SP;
    extern __shared__ float2 sm[];
    const DevJob job = a.jobs[blockIdx.x];
    const DevDomain dom = a.doms[job.dom];
    const bool vel = job.kind & JK_VEL;
    const bool ydir = job.kind & JK_Y;
    const int W = job.W;
    // strip length and field of the derivative input
    const int n = (ydir ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const long long foff = vel ? (ydir ? dom.o_vy : dom.o_vx) : dom.o_p0;
    const int pitch = vel ? (ydir ? dom.pitch_vy : dom.pitch_vx) : dom.pitch_p;
    const float* F = a.in + foff;
    const int count = job.count;
    float* smf = reinterpret_cast<float*>(sm);

    // ---- 1. gather -------------------------------------------------------
    if (!ydir) {
        // rows: pairs of rows (2cs, 2cs+1) read with 16-byte loads
        const int chunks = (n + 3) >> 2;
        for (int f = threadIdx.x; f < CS * chunks; f += NT) {
            const int cs = f / chunks, i = (f - cs * chunks) << 2;
            const int s0 = 2 * cs, s1 = s0 + 1;
            float4 u = make_float4(0.f, 0.f, 0.f, 0.f), v = u;
            const float* r0 = F + (long long)(job.first + s0) * pitch + i;
            const float* r1 = r0 + pitch;
            if (i + 4 <= n) {
                if (s0 < count) u = __ldg(reinterpret_cast<const float4*>(r0));
                if (s1 < count) v = __ldg(reinterpret_cast<const float4*>(r1));
            } else {
                if (s0 < count) { u.x = r0[0]; if (i + 1 < n) u.y = r0[1]; if (i + 2 < n) u.z = r0[2]; }
                if (s1 < count) { v.x = r1[0]; if (i + 1 < n) v.y = r1[1]; if (i + 2 < n) v.z = r1[2]; }
            }
            float2* d = sm + cs * SP + W + i;
            d[0] = make_float2(u.x, v.x);
            if (i + 1 < n) d[1] = make_float2(u.y, v.y);
            if (i + 2 < n) d[2] = make_float2(u.z, v.z);
            if (i + 3 < n) d[3] = make_float2(u.w, v.w);
        }
    } else {
        // columns: consecutive threads read consecutive columns of one row
        constexpr int S2 = 2 * CS;
        for (int f = threadIdx.x; f < S2 * n; f += NT) {
            const int s = f % S2, i = f / S2;
            float val = 0.f;
            if (s < count) val = __ldg(F + (long long)i * pitch + job.first + s);
            smf[2 * ((s >> 1) * SP + W + i) + (s & 1)] = val;
        }
    }
    // interface bands and zero padding
    {
        const float* wl = a.win + job.wtab;          // window.head(W)
        const float* wr = a.win + job.wtab + W + 1;  // window.tail(W)
        const DevDomain* D1 = job.d1 >= 0 ? &a.doms[job.d1] : nullptr;
        const DevDomain* D2 = job.d2 >= 0 ? &a.doms[job.d2] : nullptr;
        const int tail = L - 2 * W - n;
        const int per = 2 * W + tail;
        for (int f = threadIdx.x; f < 2 * CS * per; f += NT) {
            const int s = f / per, j = f - s * per;
            float val = 0.f;
            int pos;
            if (j < W) {
                pos = j;
                if (s < count && D1) {
                    const int n1 = (ydir ? D1->ny : D1->nx) + (vel ? 1 : 0);
                    const int e1 = vel ? n1 - W - 1 + j : n1 - W + j;   // far end of the low neighbour
                    const int m = vel ? W - j : W - 1 - j;              // mirrored own element
                    const float* G = a.in + (vel ? (ydir ? D1->o_vy : D1->o_vx) : D1->o_p0);
                    const int gp = vel ? (ydir ? D1->pitch_vy : D1->pitch_vx) : D1->pitch_p;
                    float raw, mir;
                    if (!ydir) {
                        raw = __ldg(G + (long long)(job.o1 + s) * gp + e1);
                        mir = __ldg(F + (long long)(job.first + s) * pitch + m);
                    } else {
                        raw = __ldg(G + (long long)e1 * gp + job.o1 + s);
                        mir = __ldg(F + (long long)m * pitch + job.first + s);
                    }
                    val = band_value(raw, mir, job.T1, job.R1, wl[j]);
                }
            } else if (j < 2 * W) {
                const int jj = j - W;
                pos = W + n + jj;
                if (s < count && D2) {
                    const int e2 = vel ? 1 + jj : jj;                   // near end of the high neighbour
                    const int m = vel ? n - 2 - jj : n - 1 - jj;
                    const float* G = a.in + (vel ? (ydir ? D2->o_vy : D2->o_vx) : D2->o_p0);
                    const int gp = vel ? (ydir ? D2->pitch_vy : D2->pitch_vx) : D2->pitch_p;
                    float raw, mir;
                    if (!ydir) {
                        raw = __ldg(G + (long long)(job.o2 + s) * gp + e2);
                        mir = __ldg(F + (long long)(job.first + s) * pitch + m);
                    } else {
                        raw = __ldg(G + (long long)e2 * gp + job.o2 + s);
                        mir = __ldg(F + (long long)m * pitch + job.first + s);
                    }
                    val = band_value(raw, mir, job.T2, job.R2, wr[jj]);
                }
            } else {
                pos = 2 * W + n + (j - 2 * W);
            }
            smf[2 * ((s >> 1) * SP + pos) + (s & 1)] = val;
        }
        // (strips beyond `count` were written as zeros by the gathers above:
        // they share complex strips with real data)
    }
    __syncthreads();

    // ---- 2-4. FFT, derivative filter, inverse FFT -------------------------
    convolve<L>(sm, a.tw, a.filt + job.dtab);
    __syncthreads();

    // ---- 5. epilogue -------------------------------------------------------
    const float cdt = a.doms[job.dom].cdt[a.stage];
    const float rho = dom.rho;
    const int nout = vel ? n - 1 : n + 1;   // cells (vel) or faces (pressure)
    if (!vel) {
        // velocity update from the pressure derivative: v = v0 - cdt * (L / rho)
        const long long vo = ydir ? dom.o_vy : dom.o_vx;
        const int vp = ydir ? dom.pitch_vy : dom.pitch_vx;
        const int ao = ydir ? dom.att_yv : dom.att_xv;
        const bool att = a.last && ao >= 0;
        if (!ydir) {
            for (int f = threadIdx.x; f < CS * nout; f += NT) {
                const int cs = f / nout, i = f - cs * nout;
                const float2 d = sm[cs * SP + W + i];
                const float dv[2] = {d.x, d.y};
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = 2 * cs + h;
                    if (s >= count) break;
                    const long long e = vo + (long long)(job.first + s) * vp + i;
                    float v = __fsub_rn(a.prev[e], __fmul_rn(cdt, __fdiv_rn(dv[h], rho)));
                    if (att) v = __fmul_rn(v, a.att[ao + i]);
                    a.out[e] = v;
                }
            }
        } else {
            constexpr int S2 = 2 * CS;
            for (int f = threadIdx.x; f < S2 * nout; f += NT) {
                const int s = f % S2, i = f / S2;
                if (s >= count) continue;
                const float dv = smf[2 * ((s >> 1) * SP + W + i) + (s & 1)];
                const long long e = vo + (long long)i * vp + job.first + s;
                float v = __fsub_rn(a.prev[e], __fmul_rn(cdt, __fdiv_rn(dv, rho)));
                if (att) v = __fmul_rn(v, a.att[ao + i]);
                a.out[e] = v;
            }
        }
    } else {
        // pressure update from the velocity derivative: p = p0 - cdt * ((L * rho) * c^2)
        const float c2 = dom.c2;
        const int pp = dom.pitch_p;
        if (!ydir) {
            for (int f = threadIdx.x; f < CS * nout; f += NT) {
                const int cs = f / nout, i = f - cs * nout;
                const float2 d = sm[cs * SP + W + i];
                const float dv[2] = {d.x, d.y};
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int s = 2 * cs + h;
                    if (s >= count) break;
                    const long long e = dom.o_px + (long long)(job.first + s) * pp + i;
                    a.out[e] = __fsub_rn(a.prev[e], __fmul_rn(cdt, __fmul_rn(__fmul_rn(dv[h], rho), c2)));
                }
            }
        } else {
            // py update, p0 = px + py (before PML), then PML on px, py at the last stage
            constexpr int S2 = 2 * CS;
            const bool last = a.last;
            for (int f = threadIdx.x; f < S2 * nout; f += NT) {
                const int s = f % S2, i = f / S2;
                if (s >= count) continue;
                const float dv = smf[2 * ((s >> 1) * SP + W + i) + (s & 1)];
                const int col = job.first + s;
                const long long e = (long long)i * pp + col;
                const float py = __fsub_rn(a.prev[dom.o_py + e], __fmul_rn(cdt, __fmul_rn(__fmul_rn(dv, rho), c2)));
                const float px = a.out[dom.o_px + e];
                a.out[dom.o_p0 + e] = __fadd_rn(px, py);
                if (last && dom.att_xp >= 0) a.out[dom.o_px + e] = __fmul_rn(px, a.att[dom.att_xp + col]);
                a.out[dom.o_py + e] = (last && dom.att_yp >= 0) ? __fmul_rn(py, a.att[dom.att_yp + i]) : py;
            }
        }
    }
}

// Carry a domain's fields through one pass unchanged (rigid domains and axes
// with should_update == false: their derivative stays zero, so the RK update
// returns the stage-start value).  The y variant also forms p0 and applies
// the PML multiply at the sixth stage, like the pass epilogue.
__global__ void copy_kernel(const DevCopy* copies, const DevDomain* doms, const float* __restrict__ prev,
                            float* __restrict__ out, const float* __restrict__ att, int last) {
    const DevCopy c = copies[blockIdx.y];
    const DevDomain d = doms[c.dom];
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (!(c.kind & JK_Y)) {
        for (int k = t0; k < d.ny * (d.nx + 1); k += stride) {
            const int r = k / (d.nx + 1), i = k - r * (d.nx + 1);
            const long long e = d.o_vx + (long long)r * d.pitch_vx + i;
            float v = prev[e];
            if (last && d.att_xv >= 0) v = __fmul_rn(v, att[d.att_xv + i]);
            out[e] = v;
        }
        for (int k = t0; k < d.ny * d.nx; k += stride) {
            const int r = k / d.nx, i = k - r * d.nx;
            const long long e = d.o_px + (long long)r * d.pitch_p + i;
            out[e] = prev[e];
        }
    } else {
        for (int k = t0; k < (d.ny + 1) * d.nx; k += stride) {
            const int r = k / d.nx, i = k - r * d.nx;
            const long long e = d.o_vy + (long long)r * d.pitch_vy + i;
            float v = prev[e];
            if (last && d.att_yv >= 0) v = __fmul_rn(v, att[d.att_yv + r]);
            out[e] = v;
        }
        for (int k = t0; k < d.ny * d.nx; k += stride) {
            const int r = k / d.nx, i = k - r * d.nx;
            const long long e = (long long)r * d.pitch_p + i;
            const float py = prev[d.o_py + e];
            const float px = out[d.o_px + e];
            out[d.o_p0 + e] = __fadd_rn(px, py);
            if (last && d.att_xp >= 0) out[d.o_px + e] = __fmul_rn(px, att[d.att_xp + i]);
            out[d.o_py + e] = (last && d.att_yp >= 0) ? __fmul_rn(py, att[d.att_yp + r]) : py;
        }
    }
}

// Gaussian speaker initial condition (kernel/core/Speaker.cpp:21-39) on every
// domain, PML included; speakers are added in order.
__global__ void speaker_kernel(const DevDomain* doms, const int* dom_x0, const int* dom_y0, const DevSpeaker* spk,
                               int n_spk, float dx, float band_width, float* set) {
    const DevDomain d = doms[blockIdx.y];
    const float x0 = (float)dom_x0[blockIdx.y], y0 = (float)dom_y0[blockIdx.y];
    const int stride = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.nx * d.ny; k += stride) {
        const int j = k / d.nx, i = k - j * d.nx;   // j: row (y), i: column (x)
        float p0 = 0.f, px = 0.f, py = 0.f;
        for (int s = 0; s < n_spk; s++) {
            const float rx = __fsub_rn(spk[s].x, x0), ry = __fsub_rn(spk[s].y, y0);
            const float ax = __fsub_rn(rx, (float)i), ay = __fsub_rn(ry, (float)j);
            // SQR(a*dx) expands to a*dx*a*dx in the reference
            const float sq = __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(ax, dx), ax), dx),
                                       __fmul_rn(__fmul_rn(__fmul_rn(ay, dx), ay), dx));
            const float p = expf(__fmul_rn(-band_width, sq));
            const float ang = atan2f(ax, ay);
            const float c = cosf(ang), sn = sinf(ang);
            p0 = __fadd_rn(p0, p);
            px = __fadd_rn(px, __fmul_rn(__fmul_rn(c, c), p));
            py = __fadd_rn(py, __fmul_rn(__fmul_rn(sn, sn), p));
        }
        const long long e = (long long)j * d.pitch_p + i;
        set[d.o_p0 + e] = p0;
        set[d.o_px + e] = px;
        set[d.o_py + e] = py;
    }
}

// One sample per receiver after the step (kernel/core/Receiver.cpp:80-83):
// p0(rel.x, rel.y) of the container, i.e. row rel.x, column rel.y.
__global__ void receiver_kernel(const DevReceiver* rec, int n_rec, const DevDomain* doms, const float* __restrict__ set,
                                float* ring, int ring_cap, int* counter) {
    const int step = *counter;
    for (int r = threadIdx.x; r < n_rec; r += blockDim.x) {
        const DevReceiver q = rec[r];
        const DevDomain d = doms[q.dom];
        ring[(long long)(step % ring_cap) * n_rec + r] = set[d.o_p0 + (long long)q.row * d.pitch_p + q.col];
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = step + 1;
}

// ---------------------------------------------------------------- host launchers
template <int L>
static cudaError_t prepare_t() {
    return cudaFuncSetAttribute(pass_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, Geo<L>::SMEM);
}

cudaError_t prepare_pass_kernels() {
    cudaError_t e;
    if ((e = prepare_t<32>()) != cudaSuccess) return e;
    if ((e = prepare_t<64>()) != cudaSuccess) return e;
    if ((e = prepare_t<128>()) != cudaSuccess) return e;
    if ((e = prepare_t<256>()) != cudaSuccess) return e;
    if ((e = prepare_t<512>()) != cudaSuccess) return e;
    if ((e = prepare_t<1024>()) != cudaSuccess) return e;
    if ((e = prepare_t<2048>()) != cudaSuccess) return e;
    if ((e = prepare_t<4096>()) != cudaSuccess) return e;
    return prepare_t<8192>();
}

template <int L>
static cudaError_t launch_pass_t(int n_jobs, const PassArgs& a, cudaStream_t st) {
    pass_kernel<L><<<n_jobs, Geo<L>::NT, Geo<L>::SMEM, st>>>(a);
    return cudaGetLastError();
}

int pass_strips_per_job(int L) {
    switch (L) {
        case 32: return 2 * Geo<32>::CS;
        case 64: return 2 * Geo<64>::CS;
        case 128: return 2 * Geo<128>::CS;
        case 256: return 2 * Geo<256>::CS;
        case 512: return 2 * Geo<512>::CS;
        case 1024: return 2 * Geo<1024>::CS;
        case 2048: return 2 * Geo<2048>::CS;
        case 4096: return 2 * Geo<4096>::CS;
        case 8192: return 2 * Geo<8192>::CS;
        default: return 0;
    }
}

// radix sequence of the in-place transform for length L (host copy of Shape<L>)
void pass_radices(int L, int* r, int* np) {
    auto set = [&](int n, int a, int b, int c, int d) { *np = n; r[0] = a; r[1] = b; r[2] = c; r[3] = d; };
    switch (L) {
        case 32: set(Shape<32>::NP, Shape<32>::R0, Shape<32>::R1, 0, 0); break;
        case 64: set(Shape<64>::NP, Shape<64>::R0, Shape<64>::R1, 0, 0); break;
        case 128: set(Shape<128>::NP, Shape<128>::R0, Shape<128>::R1, 0, 0); break;
        case 256: set(Shape<256>::NP, Shape<256>::R0, Shape<256>::R1, 0, 0); break;
        case 512: set(Shape<512>::NP, Shape<512>::R0, Shape<512>::R1, Shape<512>::R2, 0); break;
        case 1024: set(Shape<1024>::NP, Shape<1024>::R0, Shape<1024>::R1, Shape<1024>::R2, 0); break;
        case 2048: set(Shape<2048>::NP, Shape<2048>::R0, Shape<2048>::R1, Shape<2048>::R2, 0); break;
        case 4096: set(Shape<4096>::NP, Shape<4096>::R0, Shape<4096>::R1, Shape<4096>::R2, 0); break;
        case 8192: set(Shape<8192>::NP, Shape<8192>::R0, Shape<8192>::R1, Shape<8192>::R2, Shape<8192>::R3); break;
        default: *np = 0;
    }
}

cudaError_t launch_pass(int L, int n_jobs, const PassArgs& a, cudaStream_t st) {
    switch (L) {
        case 32: return launch_pass_t<32>(n_jobs, a, st);
        case 64: return launch_pass_t<64>(n_jobs, a, st);
        case 128: return launch_pass_t<128>(n_jobs, a, st);
        case 256: return launch_pass_t<256>(n_jobs, a, st);
        case 512: return launch_pass_t<512>(n_jobs, a, st);
        case 1024: return launch_pass_t<1024>(n_jobs, a, st);
        case 2048: return launch_pass_t<2048>(n_jobs, a, st);
        case 4096: return launch_pass_t<4096>(n_jobs, a, st);
        case 8192: return launch_pass_t<8192>(n_jobs, a, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_copy(const DevCopy* copies, int n, const DevDomain* doms, const float* prev, float* out,
                        const float* att, int last, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    dim3 grid(16, n);
    copy_kernel<<<grid, 256, 0, st>>>(copies, doms, prev, out, att, last);
    return cudaGetLastError();
}

cudaError_t launch_speakers(const DevDomain* doms, const int* x0, const int* y0, int n_dom, const DevSpeaker* spk,
                            int n_spk, float dx, float bw, float* set, cudaStream_t st) {
    if (n_dom <= 0) return cudaSuccess;
    dim3 grid(64, n_dom);
    speaker_kernel<<<grid, 256, 0, st>>>(doms, x0, y0, spk, n_spk, dx, bw, set);
    return cudaGetLastError();
}

cudaError_t launch_receivers(const DevReceiver* rec, int n_rec, const DevDomain* doms, const float* set, float* ring,
                             int cap, int* counter, cudaStream_t st) {
    receiver_kernel<<<1, 256, 0, st>>>(rec, n_rec, doms, set, ring, cap, counter);
    return cudaGetLastError();
}

}  // namespace pstd
