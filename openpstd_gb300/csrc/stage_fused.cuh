// stage_fused.cuh -- the fused form of the stage kernel.
//
// The same windowed Fourier derivative + RK stage update as stage_kernel
// (kernel/core/kernel_functions.cpp:123-318 fused with kernel/Solver.cpp:
// 162-182), with the strip gather folded into the first forward FFT pass and
// the RK epilogue folded into the last inverse pass:
//
//   pass A  : each thread loads the R0 positions n1 + q L/R0 of its butterfly
//             straight from global memory (p0 = px + py formed on the fly,
//             interface bands blended in place, zero padding never loaded),
//             runs the radix-R0 butterfly, applies the pass twiddles and
//             stores to the shared-memory strip;
//   middle  : the remaining forward passes, the derivative filter and the
//             first inverse passes on the shared-memory strips (shared with
//             stage_kernel; with SHF the last forward / first inverse radix
//             2H runs as a radix-2 butterfly between the two lanes of a lane
//             pair, exchanged with warp shuffles, around a radix-H butterfly
//             in registers);
//   pass A' : the last inverse pass reads its butterfly from shared memory
//             and writes the RK-updated outputs it owns straight to global
//             memory (stage-start values loaded beside it).
//
// A strip therefore crosses shared memory 2 + 2 (middle passes) times
// instead of 2 + 2 x (passes) + 2 (gather and epilogue), and every thread of
// pass A has its butterfly's loads in flight at once.  Row (x) jobs map
// consecutive lanes to consecutive positions of one strip pair (128-byte
// coalesced row loads); column (y) jobs map consecutive lanes to the strip
// pairs first (adjacent columns of the same rows, 8-byte loads).
#pragma once
#include "stage_kernel.cuh"

namespace pstd {

// Fused-form configuration: Cfg's geometry plus SHF (the last radix, 2H, is
// split across a lane pair with shuffles).  The first pass needs L/R0 >= 16
// so that a row job's half-warp reads 64 contiguous bytes.
template <int L_, int CS_, int NT_, int MINB_, int R0_, int R1_, int R2_ = 0, int R3_ = 0, int SHF_ = 0>
struct FCfg : Cfg<L_, CS_, NT_, MINB_, R0_, R1_, R2_, R3_> {
    static constexpr int SHF = SHF_;
    static_assert(L_ / R0_ >= 16, "first pass too wide for coalesced row loads");
    // shared memory: the strips, then the blended interface bands of every
    // real strip (2 x 32 floats: windows are at most 32 wide)
    static constexpr int BAND = 64;
    static constexpr int FSMEM = Cfg<L_, CS_, NT_, MINB_, R0_, R1_, R2_, R3_>::BUF * 8 + 2 * CS_ * BAND * 4;
};

__device__ __forceinline__ float2 ldf2(const float* p) {   // p 8-byte aligned
    float2 v;
    asm("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
}

// The neighbours of one job: their strip sources and the length of d1's strips.
struct FusedBands {
    Src S1, S3;
    int nl1;
    const float* wl;   // window.head(W)
    const float* wr;   // window.tail(W)
};

__device__ __forceinline__ FusedBands fused_bands(const StageArgs& A, const DevJob& job, bool vel, bool ydir,
                                                  bool first) {
    FusedBands b;
    b.S1 = Src{nullptr, nullptr, 0};
    b.S3 = Src{nullptr, nullptr, 0};
    b.nl1 = 0;
    if (job.d1 >= 0) {
        const DevDomain D1 = A.doms[job.d1];
        b.S1 = strip_source(A, D1, vel, ydir, first);
        b.nl1 = (ydir ? D1.ny : D1.nx) + (vel ? 1 : 0);
    }
    if (job.d2 >= 0) b.S3 = strip_source(A, A.doms[job.d2], vel, ydir, first);
    b.wl = A.win + job.wtab;
    b.wr = A.win + job.wtab + job.W + 1;
    return b;
}

// Band value of real strip s at transform position p (p < W: the low band,
// else the high band, p in [W+n, 2W+n)), in the reference's operation order
// (kernel/core/kernel_functions.cpp:191-216 for pressure, :246-269 for velocity).
template <bool YDIR, bool VEL>
__device__ __forceinline__ float fused_band(const DevJob& job, const Src& S, const FusedBands& B, int n, int s, int p) {
    const int W = job.W;
    if (p < W) {
        if (job.d1 < 0) return 0.f;
        const int e1 = VEL ? B.nl1 - W - 1 + p : B.nl1 - W + p;   // far end of the low neighbour
        const int m = VEL ? W - p : W - 1 - p;                      // mirrored own element
        const float raw = YDIR ? B.S1.at((long long)e1 * B.S1.pitch + job.o1 + s)
                               : B.S1.at((long long)(job.o1 + s) * B.S1.pitch + e1);
        const float mir = YDIR ? S.at((long long)m * S.pitch + job.first + s) : S.at((long long)(job.first + s) * S.pitch + m);
        return band_value(raw, mir, job.T1, job.R1, __ldg(B.wl + p));
    }
    if (job.d2 < 0) return 0.f;
    const int jj = p - W - n;
    const int e2 = VEL ? 1 + jj : jj;                  // near end of the high neighbour
    const int m = VEL ? n - 2 - jj : n - 1 - jj;
    const float raw = YDIR ? B.S3.at((long long)e2 * B.S3.pitch + job.o2 + s)
                           : B.S3.at((long long)(job.o2 + s) * B.S3.pitch + e2);
    const float mir = YDIR ? S.at((long long)m * S.pitch + job.first + s) : S.at((long long)(job.first + s) * S.pitch + m);
    return band_value(raw, mir, job.T2, job.R2, __ldg(B.wr + jj));
}

// twiddles of the first pass (table offset 0): x[k] *= w[n1][k] (INV: conjugate)
template <int R, bool INV>
__device__ __forceinline__ void first_twiddles(float2 (&x)[R], const float2* tw, int n1) {
    const float4* t4 = reinterpret_cast<const float4*>(tw + n1 * R);
#pragma unroll
    for (int h = 0; h < R / 2; h++) {
        const float4 v = __ldg(t4 + h);
        if (h) x[2 * h] = INV ? cmulc(x[2 * h], make_float2(v.x, v.y)) : cmul(x[2 * h], make_float2(v.x, v.y));
        x[2 * h + 1] = INV ? cmulc(x[2 * h + 1], make_float2(v.z, v.w)) : cmul(x[2 * h + 1], make_float2(v.z, v.w));
    }
}

// ---- pass A: gather + first forward pass
// sband: the job's blended bands, written here by every thread before the
// barrier that precedes their use (the barrier is taken inside).
template <class C, int NTH, bool YDIR, bool VEL, bool TWO>
__device__ __forceinline__ void fused_first(float2* sm, float* sband, const StageArgs& A, const DevJob& job,
                                            const DevDomain& dom, const Src& S, bool first, int tid) {
    constexpr int R = C::R0, Q = C::L / R, CS = C::CS, SP = C::SP, S2 = 2 * CS, BAND = C::BAND;
    constexpr int ITEMS = CS * Q;
    static_assert(ITEMS <= NTH * 4, "at most four butterflies per thread");
    const int W = job.W;
    const int n = (YDIR ? dom.ny : dom.nx) + (VEL ? 1 : 0);
    const int count = job.count;
    // band values: S2 x 2W per job, at most two per thread in flight
    constexpr int BPT = (S2 * BAND + NTH - 1) / NTH;
    float bv[BPT];
    {
        const FusedBands B = fused_bands(A, job, VEL, YDIR, first);
#pragma unroll
        for (int k = 0; k < BPT; k++) {
            const int idx = tid + k * NTH;
            const int s = idx / (2 * W), j = idx - s * (2 * W);
            bv[k] = 0.f;
            if (s < count && idx < S2 * 2 * W) bv[k] = fused_band<YDIR, VEL>(job, S, B, n, s, j < W ? j : n + j);
        }
    }
    const bool even = !(job.first & 1);   // column pairs 8-byte aligned
    constexpr int NIT = (ITEMS + NTH - 1) / NTH;
    float2 x[NIT][R];
#pragma unroll
    for (int t = 0; t < NIT; t++) {
        const int it = tid + t * NTH;
        const int cs = YDIR ? it % CS : it / Q;
        const int n1 = YDIR ? it / CS : it % Q;
        const int s0 = 2 * cs;
        const bool h0 = it < ITEMS && s0 < count, h1 = it < ITEMS && s0 + 1 < count;
        if (!YDIR) {
            const long long r0 = (long long)(job.first + s0) * S.pitch;
            const float* a0 = S.a + r0 - W;
            const float* b0 = TWO ? S.b + r0 - W : nullptr;
            const int P = S.pitch;
#pragma unroll
            for (int q = 0; q < R; q++) {
                const int p = n1 + q * Q;
                const bool in = p >= W && p < W + n;
                float re = 0.f, im = 0.f;
                if (in && h0) re = TWO ? __fadd_rn(ldf(a0 + p), ldf(b0 + p)) : ldf(a0 + p);
                if (in && h1) im = TWO ? __fadd_rn(ldf(a0 + P + p), ldf(b0 + P + p)) : ldf(a0 + P + p);
                x[t][q] = make_float2(re, im);
            }
        } else {
            const long long c0 = job.first + s0 - (long long)W * S.pitch;
            const float* a0 = S.a + c0;
            const float* b0 = TWO ? S.b + c0 : nullptr;
            const long long P = S.pitch;
#pragma unroll
            for (int q = 0; q < R; q++) {
                const int p = n1 + q * Q;
                const bool in = p >= W && p < W + n && h0;
                float2 v = make_float2(0.f, 0.f);
                if (in) {
                    const long long e = (long long)p * P;
                    if (even && h1) {
                        v = ldf2(a0 + e);
                        if (TWO) {
                            const float2 u = ldf2(b0 + e);
                            v = make_float2(__fadd_rn(v.x, u.x), __fadd_rn(v.y, u.y));
                        }
                    } else {
                        v.x = TWO ? __fadd_rn(ldf(a0 + e), ldf(b0 + e)) : ldf(a0 + e);
                        if (h1) v.y = TWO ? __fadd_rn(ldf(a0 + e + 1), ldf(b0 + e + 1)) : ldf(a0 + e + 1);
                    }
                }
                x[t][q] = v;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < BPT; k++) {
        const int idx = tid + k * NTH;
        if (idx < S2 * 2 * W) sband[(idx / (2 * W)) * BAND + idx % (2 * W)] = bv[k];
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < NIT; t++) {
        const int it = tid + t * NTH;
        if (it >= ITEMS) break;
        const int cs = YDIR ? it % CS : it / Q;
        const int n1 = YDIR ? it / CS : it % Q;
        const int s0 = 2 * cs;
        // interface bands, positions [0, W) and [W+n, 2W+n): the tests on q
        // are uniform over the block, the position tests per thread
#pragma unroll
        for (int q = 0; q < R; q++) {
            const int p = n1 + q * Q;
            const bool lo_q = q * Q < W;
            const bool hi_q = (q + 1) * Q > W + n && q * Q < 2 * W + n;
            if (lo_q || hi_q) {
                if (p < W || (p >= W + n && p < 2 * W + n)) {
                    const int j = p < W ? p : p - n;
                    x[t][q] = make_float2(sband[s0 * BAND + j], sband[(s0 + 1) * BAND + j]);
                }
            }
        }
        DFT<R, false>::run(x[t]);
        first_twiddles<R, false>(x[t], A.tw, n1);
        float2* base = sm + cs * SP + n1;
#pragma unroll
        for (int k = 0; k < R; k++) base[k * Q] = x[t][k];
    }
}

// ---- pass A': last inverse pass + RK update (+ PML multiply of vx / vy at
// the sixth stage), outputs [W, W + nout) of every strip
template <class C, int NTH, bool YDIR, bool VEL, bool ATT>
__device__ __forceinline__ void fused_last(const float2* sm, const StageArgs& A, const DevJob& job, const DevDomain& dom,
                                           int tid) {
    constexpr int R = C::R0, Q = C::L / R, CS = C::CS, SP = C::SP;
    constexpr int ITEMS = CS * Q;
    constexpr int CH = R < 8 ? R : 8;   // outputs whose stage-start values are in flight together
    const float* __restrict__ prev = A.prev;
    float* __restrict__ out = A.out;
    const int W = job.W;
    const int n = (YDIR ? dom.ny : dom.nx) + (VEL ? 1 : 0);
    const int nout = VEL ? n - 1 : n + 1;   // cells (vel) or faces (pressure)
    const int count = job.count;
    const float cdt = A.doms[job.dom].cdt[A.stage];
    const float rho = dom.rho, c2 = dom.c2, rinv = __frcp_rn(rho);
    long long fo;
    int fp, ao;
    if (!VEL) {
        fo = YDIR ? dom.o_vy : dom.o_vx;
        fp = YDIR ? dom.pitch_vy : dom.pitch_vx;
        ao = YDIR ? dom.att_yv : dom.att_xv;
    } else {
        fo = YDIR ? dom.o_py : dom.o_px;
        fp = dom.pitch_p;
        ao = -1;
    }
    const bool even = !(job.first & 1);
    for (int it = tid; it < ITEMS; it += NTH) {
        const int cs = YDIR ? it % CS : it / Q;
        const int n1 = YDIR ? it / CS : it % Q;
        const int s0 = 2 * cs;
        if (s0 >= count) continue;
        const bool h1 = s0 + 1 < count;
        const float2* base = sm + cs * SP + n1;
        float2 x[R];
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = base[k * Q];
        first_twiddles<R, true>(x, A.tw, n1);
        DFT<R, true>::run(x);
        long long e0;
        if (!YDIR) e0 = fo + (long long)(job.first + s0) * fp - W;
        else e0 = fo + job.first + s0 - (long long)W * fp;
#pragma unroll
        for (int c = 0; c < R; c += CH) {
            float2 pv[CH];
#pragma unroll
            for (int u = 0; u < CH; u++) {
                const int p = n1 + (c + u) * Q;
                float2 v = make_float2(0.f, 0.f);
                if (p >= W && p < W + nout) {
                    if (!YDIR) {
                        v.x = ldf(prev + e0 + p);
                        if (h1) v.y = ldf(prev + e0 + fp + p);
                    } else {
                        const long long e = e0 + (long long)p * fp;
                        if (even && h1) v = ldf2(prev + e);
                        else {
                            v.x = ldf(prev + e);
                            if (h1) v.y = ldf(prev + e + 1);
                        }
                    }
                }
                pv[u] = v;
            }
#pragma unroll
            for (int u = 0; u < CH; u++) {
                const int p = n1 + (c + u) * Q;
                if (p < W || p >= W + nout) continue;
                float v0 = rk_update(pv[u].x, x[c + u].x, VEL, cdt, rho, c2, rinv);
                float v1 = rk_update(pv[u].y, x[c + u].y, VEL, cdt, rho, c2, rinv);
                if (ATT) {
                    const float a = __ldg(A.att + ao + (p - W));
                    v0 = __fmul_rn(v0, a);
                    v1 = __fmul_rn(v1, a);
                }
                if (!YDIR) {
                    out[e0 + p] = v0;
                    if (h1) out[e0 + fp + p] = v1;
                } else {
                    const long long e = e0 + (long long)p * fp;
                    if (even && h1) {
                        *reinterpret_cast<float2*>(out + e) = make_float2(v0, v1);
                    } else {
                        out[e] = v0;
                        if (h1) out[e + 1] = v1;
                    }
                }
            }
        }
    }
}

// ---- middle radix 2H as a lane-pair radix-2 butterfly around a radix-H one
// A block of 2H contiguous positions (one DFT of the last forward pass) is
// held by a lane pair, lane h holding positions h H + j.  Forward:
//   a_j = x_j + x_{j+H}  (lane 0),   b_j = (x_j - x_{j+H}) W^j  (lane 1),
//   W = exp(-2 pi i / 2H); DFT_H over j then gives bin 2k + h in register k.
// After the filter (position 2k + h of the block in the table) and the inverse
// DFT_H, the inverse radix-2 is x_j = a'_j + conj(W^j) b'_j,
// x_{j+H} = a'_j - conj(W^j) b'_j.  The lane-pair exchanges are warp shuffles
// (two per complex value and direction); the twiddle table holds 2H entries,
// 1 for lane 0 and W^j for lane 1, so both lanes run the same instructions.
template <class C, int H, int NTH>
__device__ __forceinline__ void mid_pass_shf(float2* sm, const float2* filt, const float2* tws, int tid) {
    constexpr int ITEMS = C::CS * (C::L / (2 * H)) * 2;
    static_assert(ITEMS % 32 == 0 && NTH % 32 == 0, "whole warps take part in the exchanges");
    const int h = tid & 1;
    const float sg = h ? -1.f : 1.f;
    const float4* t4 = reinterpret_cast<const float4*>(tws + h * H);
    for (int it = tid; it < ITEMS; it += NTH) {
        const int pair = it >> 1;
        const int cs = pair % C::CS, blk = pair / C::CS;
        float2* base = sm + cs * C::SP + blk * (2 * H) + h * H;
        float2 x[H];
        // 16-byte accesses need an even strip pitch (every strip 16-byte aligned)
        if constexpr (C::SP % 2 == 0) {
#pragma unroll
            for (int j = 0; j < H / 2; j++) {
                const float4 v = reinterpret_cast<const float4*>(base)[j];
                x[2 * j] = make_float2(v.x, v.y);
                x[2 * j + 1] = make_float2(v.z, v.w);
            }
        } else {
#pragma unroll
            for (int j = 0; j < H; j++) x[j] = base[j];
        }
#pragma unroll
        for (int j = 0; j < H; j++) {
            const float yx = __shfl_xor_sync(0xffffffffu, x[j].x, 1);
            const float yy = __shfl_xor_sync(0xffffffffu, x[j].y, 1);
            // lane 0: x + y; lane 1: y - x
            x[j] = make_float2(__fmaf_rn(sg, x[j].x, yx), __fmaf_rn(sg, x[j].y, yy));
        }
#pragma unroll
        for (int j = 0; j < H / 2; j++) {
            const float4 w = __ldg(t4 + j);
            x[2 * j] = cmul(x[2 * j], make_float2(w.x, w.y));
            x[2 * j + 1] = cmul(x[2 * j + 1], make_float2(w.z, w.w));
        }
        DFT<H, false>::run(x);
        const float2* f = filt + blk * (2 * H) + h;
#pragma unroll
        for (int k = 0; k < H; k++) x[k] = cmul(x[k], __ldg(f + 2 * k));
        DFT<H, true>::run(x);
#pragma unroll
        for (int j = 0; j < H / 2; j++) {
            const float4 w = __ldg(t4 + j);
            x[2 * j] = cmulc(x[2 * j], make_float2(w.x, w.y));
            x[2 * j + 1] = cmulc(x[2 * j + 1], make_float2(w.z, w.w));
        }
#pragma unroll
        for (int j = 0; j < H; j++) {
            const float yx = __shfl_xor_sync(0xffffffffu, x[j].x, 1);
            const float yy = __shfl_xor_sync(0xffffffffu, x[j].y, 1);
            // lane 0: a' + c; lane 1: a' - c  (lane 0 holds a', lane 1 holds c)
            x[j] = make_float2(__fmaf_rn(sg, x[j].x, yx), __fmaf_rn(sg, x[j].y, yy));
        }
        if constexpr (C::SP % 2 == 0) {
#pragma unroll
            for (int j = 0; j < H / 2; j++)
                reinterpret_cast<float4*>(base)[j] = make_float4(x[2 * j].x, x[2 * j].y, x[2 * j + 1].x, x[2 * j + 1].y);
        } else {
#pragma unroll
            for (int j = 0; j < H; j++) base[j] = x[j];
        }
    }
}

template <class C, int R, int NTH>
__device__ __forceinline__ void fused_mid_radix(float2* sm, const float2* tw, const float2* filt, int tid) {
    if constexpr (C::SHF) mid_pass_shf<C, R / 2, NTH>(sm, filt, tw + C::TWN, tid);
    else mid_pass<C, R, NTH, false>(sm, filt, tid);
}

// the passes between pass A and pass A'
template <class C, int NTH>
__device__ __forceinline__ void fused_middle(float2* sm, const float2* tw, const float2* filt, int tid) {
    constexpr int M1 = C::M1, M2 = C::M2;
    constexpr int T1 = C::T1, T2 = C::T2;
    if constexpr (C::NP == 2) {
        fused_mid_radix<C, C::R1, NTH>(sm, tw, filt, tid);
    } else if constexpr (C::NP == 3) {
        fwd_pass<C, C::R1, M1, T1, NTH, false>(sm, tw, tid);
        __syncthreads();
        fused_mid_radix<C, C::R2, NTH>(sm, tw, filt, tid);
        __syncthreads();
        inv_pass<C, C::R1, M1, T1, NTH, false>(sm, tw, tid);
    } else {
        fwd_pass<C, C::R1, M1, T1, NTH, false>(sm, tw, tid);
        __syncthreads();
        fwd_pass<C, C::R2, M2, T2, NTH, false>(sm, tw, tid);
        __syncthreads();
        fused_mid_radix<C, C::R3, NTH>(sm, tw, filt, tid);
        __syncthreads();
        inv_pass<C, C::R2, M2, T2, NTH, false>(sm, tw, tid);
        __syncthreads();
        inv_pass<C, C::R1, M1, T1, NTH, false>(sm, tw, tid);
    }
}

template <class C, int NTH>
__device__ __forceinline__ void fused_gather(float2* sm, float* sband, const StageArgs& A, const DevJob& job,
                                             const DevDomain& dom, bool first, int tid) {
    const bool vel = job.kind & JK_VEL, ydir = job.kind & JK_Y;
    const Src S = strip_source(A, dom, vel, ydir, first);
    if (vel) {
        if (ydir) fused_first<C, NTH, true, true, false>(sm, sband, A, job, dom, S, first, tid);
        else fused_first<C, NTH, false, true, false>(sm, sband, A, job, dom, S, first, tid);
    } else if (S.b) {
        if (ydir) fused_first<C, NTH, true, false, true>(sm, sband, A, job, dom, S, first, tid);
        else fused_first<C, NTH, false, false, true>(sm, sband, A, job, dom, S, first, tid);
    } else {
        if (ydir) fused_first<C, NTH, true, false, false>(sm, sband, A, job, dom, S, first, tid);
        else fused_first<C, NTH, false, false, false>(sm, sband, A, job, dom, S, first, tid);
    }
}

template <class C, int NTH>
__device__ __forceinline__ void fused_epilogue(const float2* sm, const StageArgs& A, const DevJob& job,
                                               const DevDomain& dom, int tid) {
    const bool ydir = job.kind & JK_Y;
    if (job.kind & JK_VEL) {
        if (ydir) fused_last<C, NTH, true, true, false>(sm, A, job, dom, tid);
        else fused_last<C, NTH, false, true, false>(sm, A, job, dom, tid);
        return;
    }
    const int ao = ydir ? dom.att_yv : dom.att_xv;
    if (A.last && ao >= 0) {
        if (ydir) fused_last<C, NTH, true, false, true>(sm, A, job, dom, tid);
        else fused_last<C, NTH, false, false, true>(sm, A, job, dom, tid);
    } else {
        if (ydir) fused_last<C, NTH, true, false, false>(sm, A, job, dom, tid);
        else fused_last<C, NTH, false, false, false>(sm, A, job, dom, tid);
    }
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_fused(StageArgs A) {
    extern __shared__ __align__(16) float2 sm[];
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    if (job.kind & JK_COPY) {
        copy_axis<C::NT>(A, dom, job.kind & JK_Y, threadIdx.x);
        return;
    }
    const bool first = A.first_step[dom.scene] != 0;
    fused_gather<C, C::NT>(sm, reinterpret_cast<float*>(sm + C::BUF), A, job, dom, first, threadIdx.x);
    __syncthreads();
    fused_middle<C, C::NT>(sm, A.tw, A.filt + job.dtab, threadIdx.x);
    __syncthreads();
    fused_epilogue<C, C::NT>(sm, A, job, dom, threadIdx.x);
}

template <class C>
cudaError_t launch_fused_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    stage_fused<C><<<n_jobs, C::NT, C::FSMEM, st>>>(a);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_fused_t() {
    return cudaFuncSetAttribute(stage_fused<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::FSMEM);
}

template <class C>
size_t fused_smem(int) {
    return (size_t)C::FSMEM;
}

template <class C>
StageVariant make_fused_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT; v.smem = C::FSMEM; v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.persistent = false;
    v.pipe = false;
    v.bf16 = false;
    v.shf = C::SHF;
    v.launch = &launch_fused_t<C>;
    v.prepare = &prepare_fused_t<C>;
    v.smem_for = &fused_smem<C>;
    v.name = name;
    return v;
}

}  // namespace pstd
