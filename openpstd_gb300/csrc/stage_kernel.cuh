// stage_kernel.cuh -- one RK stage of the strip-derivative solve, sm_103a.
//
// A job is up to 2*CS adjacent strips (rows for x, columns for y) of one
// domain sharing both interface neighbours.  For each strip the kernels
// compute the reference's windowed Fourier derivative (kernel/core/
// kernel_functions.cpp:123-318) fused with the RK stage update
// (kernel/Solver.cpp:162-182):
//
//   1. gather: strip + the two W-wide interface bands of the neighbours
//      (reflected / transmitted and windowed, kernel/core/kernel_functions.cpp:
//      191-216,246-269), zero padded to L, two real strips per complex strip,
//      in shared memory; p0 is formed as px + py of the previous stage while
//      loading;
//   2. forward complex FFT of length L in place (decimation in frequency,
//      radix 16/8/4/2 butterflies in registers, per-pass twiddle tables built
//      in FP64), output in digit-reversed position order;
//   3. multiply by the Hermitian-extended derivative filter i k e^{-/+ i k dx/2}
//      (1/L folded in) stored in the same position order, fused with the last
//      forward and the first inverse pass;
//   4. inverse FFT (decimation in time), natural order;
//   5. epilogue: slice W..W+n and RK-update against the stage-start set
//      (vx/vy get the PML multiply of the sixth stage here).
//
// Two kernel forms share these steps:
//   stage_kernel  -- one CTA per job, all threads do every step;
//   stage_ws      -- persistent and warp specialised: per SM one CTA walks a
//                    list of jobs; memory warps gather job j+1 and write back
//                    job j-1 while FFT warps transform job j (two shared-
//                    memory buffers handed over with named barriers); the
//                    twiddle tables and both derivative filters are staged in
//                    shared memory once per CTA;
//   stage_pipe    -- persistent, all warps do every step; the strips, bands
//                    and stage-start values of job k+2 are copied to shared
//                    memory with cp.async while job k is transformed.
// The autotuner times every form on the bucket's own jobs and keeps the
// fastest (the pipelined form wins for the short PML-normal strips).
//
// Packing two real strips into one complex strip is exact in real
// arithmetic: the filter is Hermitian, so the operator is real and acts on
// the real and imaginary parts separately.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "launch.hpp"
#include "transform_gain.hpp"

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

// cos / sin of multiples of pi/8 and pi/16: PSTD_C8 .. PSTD_S316 (transform_gain.hpp)

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

// a * exp(-/+ 2 pi i K / 32); odd K use cos / sin of multiples of pi/16
template <int K, bool INV>
__device__ __forceinline__ float2 tw32(float2 a) {
    constexpr float sg = INV ? 1.f : -1.f;
    if constexpr ((K & 1) == 0) {
        return tw16<K / 2, INV>(a);
    } else {
        constexpr float c = K == 1 ? PSTD_C16 : K == 3 ? PSTD_C316 : K == 5 ? PSTD_S316 : K == 7 ? PSTD_S16
                          : K == 9 ? -PSTD_S16 : K == 11 ? -PSTD_S316 : K == 13 ? -PSTD_C316 : -PSTD_C16;
        constexpr float s = K == 1 ? PSTD_S16 : K == 3 ? PSTD_S316 : K == 5 ? PSTD_C316 : K == 7 ? PSTD_C16
                          : K == 9 ? PSTD_C16 : K == 11 ? PSTD_C316 : K == 13 ? PSTD_S316 : PSTD_S16;
        return cmul(a, make_float2(c, sg * s));
    }
}

template <int K, bool INV>
__device__ __forceinline__ void tw32_all(float2* o) {
    if constexpr (K < 16) {
        o[K] = tw32<K, INV>(o[K]);
        tw32_all<K + 1, INV>(o);
    }
}

template <bool INV>
struct DFT<32, INV> {
    static __device__ __forceinline__ void run(float2* x) {
        float2 e[16], o[16];
#pragma unroll
        for (int k = 0; k < 16; k++) { e[k] = x[2 * k]; o[k] = x[2 * k + 1]; }
        DFT<16, INV>::run(e);
        DFT<16, INV>::run(o);
        tw32_all<1, INV>(o);
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x[k] = cadd(e[k], o[k]);
            x[k + 16] = csub(e[k], o[k]);
        }
    }
};

// Computed twiddles: float2 read per butterfly for radix R -- (w, w^2, w^4,
// w^8) for R = 16, (w, w^4) for R = 8, (w, w^2) for R = 4, (w, w) for R = 2;
// the rest are products of at most three of them (make_twiddles).
__host__ __device__ constexpr int tw_entry(int R) { return R >= 16 ? 4 : 2; }

// ---------------------------------------------------------------- variants
// Plain form: L, complex strips per CTA, threads, min CTAs per SM, radices.
// Persistent form (NTP > 0): NT FFT threads + NTP memory threads.
// TC = 1: radix-16 passes as split-BF16 tensor-core GEMMs (precision study).
// ILP = 1: the transform passes load two butterflies before computing either
// (shared-memory stores of one butterfly do not hold back the other's loads).
// CTW = 1: the twiddles of a pass are formed in registers from a few powers
// read from the table (tw_entry below) instead of read one by one: the
// table loads through L1 were the largest share of the transform passes' L1
// traffic.
template <int L_, int CS_, int NT_, int MINB_, int R0_, int R1_, int R2_ = 0, int R3_ = 0, int NTP_ = 0, int TC_ = 0,
          int ILP_ = 0, int CTW_ = 0>
struct Cfg {
    static constexpr int L = L_, CS = CS_, NT = NT_, MINB = MINB_, NTP = NTP_, TC = TC_, ILP = ILP_, CTW = CTW_;
    static constexpr int R0 = R0_, R1 = R1_, R2 = R2_, R3 = R3_;
    static constexpr int NP = R3_ ? 4 : (R2_ ? 3 : 2);
    static_assert(R0 * R1 * (R2 ? R2 : 1) * (R3 ? R3 : 1) == L, "radix plan must multiply to L");
    // strip pitch in float2: L + 16/CS (mod 16), so that the CS strips a
    // half-warp touches at one offset fall in distinct bank pairs
    static constexpr int PAD = CS >= 16 ? 1 : 16 / CS;
    static constexpr int SP = L + PAD;
    static constexpr int BUF = CS * SP;            // float2 per job buffer
    // twiddle table: one [n1][k] block of M entries per pass but the last
    static constexpr int M1 = L / R0, M2 = M1 / R1;
    // float2 per butterfly row of a pass's table: R (one per twiddle) or, with
    // CTW, the powers tw_entry<R>() lists
    static constexpr int TE0 = CTW ? tw_entry(R0) : R0, TE1 = CTW ? tw_entry(R1) : R1, TE2 = CTW ? tw_entry(R2 ? R2 : 1) : R2;
    static constexpr int T1 = (L / R0) * TE0;                   // offset of pass 1's table
    static constexpr int T2 = T1 + (M1 / R1) * TE1;             // offset of pass 2's table
    static constexpr int TWN = NP == 2 ? T1 : (NP == 3 ? T2 : T2 + (R2 ? (M2 / R2) * TE2 : 0));
    static constexpr int SMEM = NTP ? (2 * BUF + TWN + 2 * L) * 8 : BUF * 8;
};

// group-local barrier: BAR 0 = the whole CTA, else a named barrier of NTH threads
template <int BAR, int NTH>
__device__ __forceinline__ void group_sync() {
    if constexpr (BAR == 0) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"n"(BAR), "n"(NTH) : "memory");
}
__device__ __forceinline__ void bar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void bar_arrive(int id, int n) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory"); }

template <bool SMT, class T>
__device__ __forceinline__ T tload(const T* p) {   // table load: shared (SMT) or read-only global
    if constexpr (SMT) return *p;
    else return __ldg(p);
}

// Twiddles of a pass with block size M and radix R: table [n1][k] =
// exp(-2 pi i n1 k / M), n1 < M/R, k < R (k = 0 included, so a row is R
// float2 read as R/2 16-byte loads).
template <int R, bool SMT>
__device__ __forceinline__ void load_twiddles(const float2* row, float2 (&w)[R]) {
    const float4* t4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int h = 0; h < R / 2; h++) {
        const float4 v = tload<SMT>(t4 + h);
        w[2 * h] = make_float2(v.x, v.y);
        w[2 * h + 1] = make_float2(v.z, v.w);
    }
}

// w[k] = w^k, k < R, from the row of powers tw_entry<R> lists (FP64-built);
// no product chains more than three roundings
template <int R, bool SMT>
__device__ __forceinline__ void make_twiddles(const float2* row, float2 (&w)[R]) {
    const float4* t4 = reinterpret_cast<const float4*>(row);
    const float4 a = tload<SMT>(t4);
    const float2 w1 = make_float2(a.x, a.y), wb = make_float2(a.z, a.w);
    w[0] = make_float2(1.f, 0.f);
    if constexpr (R == 2) {
        w[1] = w1;
    } else if constexpr (R == 4) {
        w[1] = w1;
        w[2] = wb;
        w[3] = cmul(wb, w1);
    } else if constexpr (R == 8) {
        const float2 w2 = cmul(w1, w1), w3 = cmul(w2, w1);
        w[1] = w1; w[2] = w2; w[3] = w3; w[4] = wb;
        w[5] = cmul(wb, w1); w[6] = cmul(wb, w2); w[7] = cmul(wb, w3);
    } else {
        static_assert(R == 16, "computed twiddles for radix 2..16");
        const float4 b = tload<SMT>(t4 + 1);
        const float2 w2 = wb, w4 = make_float2(b.x, b.y), w8 = make_float2(b.z, b.w);
        const float2 w3 = cmul(w2, w1), w12 = cmul(w8, w4);
        w[1] = w1; w[2] = w2; w[3] = w3; w[4] = w4;
        w[5] = cmul(w4, w1); w[6] = cmul(w4, w2); w[7] = cmul(w4, w3); w[8] = w8;
        w[9] = cmul(w8, w1); w[10] = cmul(w8, w2); w[11] = cmul(w8, w3); w[12] = w12;
        w[13] = cmul(w12, w1); w[14] = cmul(w12, w2); w[15] = cmul(w12, w3);
    }
}

template <class C, int R, bool SMT>
__device__ __forceinline__ void pass_twiddles(const float2* tab, int n1, float2 (&w)[R]) {
    if constexpr (C::CTW) make_twiddles<R, SMT>(tab + n1 * tw_entry(R), w);
    else load_twiddles<R, SMT>(tab + n1 * R, w);
}

// ---------------------------------------------------------------- split-BF16 DFT-16 on tensor cores
// Precision study for long strips (an opt-in variant, never picked by the
// autotuner): sixteen radix-16 butterflies of a pass form the rows of a real
// GEMM  [Re x | Im x] (16 x 32) * F (32 x 32) = [Re y | Im y]  with
// F = [[C, -S], [S, C]], C = cos(2 pi q k / 16), S = sin(...) for the
// forward transform (the inverse flips the sign of the S blocks).  Every
// operand is split into bf16 hi + lo (x = hi + lo to about 2^-17), and the
// product is accumulated in fp32 as lo*hi + hi*lo + hi*hi (lo*lo dropped) on
// mma.sync m16n8k16 (row.col, bf16 -> f32).  Lane (g = lane / 4, t = lane % 4)
// holds two butterflies (rows g and g + 8) at the positions {2t, 2t+1, 2t+8,
// 2t+9}; the accumulator layout of m16n8 equals the A layout of the next
// product, so forward DFT -> filter -> inverse DFT stays in registers.

__device__ __forceinline__ float cos16(int m) {   // cos(2 pi m / 16)
    switch (m & 15) {
        case 0: return 1.f;
        case 1: case 15: return PSTD_C8;
        case 2: case 14: return PSTD_R2;
        case 3: case 13: return PSTD_S8;
        case 4: case 12: return 0.f;
        case 5: case 11: return -PSTD_S8;
        case 6: case 10: return -PSTD_R2;
        case 7: case 9: return -PSTD_C8;
        default: return -1.f;
    }
}
__device__ __forceinline__ float sin16(int m) { return cos16(m - 4); }   // sin(x) = cos(x - pi/2)

__device__ __forceinline__ void split_pack(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);   // a in the low half (lower column)
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// B fragments of the forward matrix: [kk][nt][reg], k = kk*16 + 2t + 8*reg (+1), n = nt*8 + g
struct TCFrag {
    uint32_t hi[2][4][2], lo[2][4][2];
};

__device__ __forceinline__ float dft_entry_fwd(int k, int n) {
    const int m = ((k & 15) * (n & 15)) & 15;
    const bool xi = k >= 16, yi = n >= 16;
    if (xi == yi) return cos16(m);
    return xi ? sin16(m) : -sin16(m);
}

__device__ __forceinline__ void tc_matrix(TCFrag& F, int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kk = 0; kk < 2; kk++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int k = kk * 16 + 2 * t + 8 * r, n = nt * 8 + g;
                split_pack(dft_entry_fwd(k, n), dft_entry_fwd(k + 1, n), F.hi[kk][nt][r], F.lo[kk][nt][r]);
            }
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// positions of the lane's four values within a butterfly: 2t, 2t+1, 2t+8, 2t+9
__device__ __forceinline__ int tc_pos(int t, int j) { return 2 * t + (j & 1) + ((j >> 1) << 3); }

// y = DFT16(x) (INV: inverse, unnormalised) for the lane's two butterflies
template <bool INV>
__device__ __forceinline__ void tc_dft(const float2 (&x)[2][4], float2 (&y)[2][4], const TCFrag& F) {
    uint32_t ah[2][4], al[2][4];
#pragma unroll
    for (int kk = 0; kk < 2; kk++) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            // a regs: 0 (row g, cols 2t..), 1 (row g+8), 2 (row g, cols 2t+8..), 3 (row g+8, cols 2t+8..)
            const int i = r & 1, j = (r >> 1) * 2;
            const float2 u = x[i][j], v = x[i][j + 1];
            split_pack(kk ? u.y : u.x, kk ? v.y : v.x, ah[kk][r], al[kk][r]);
        }
    }
    float d[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
#pragma unroll
        for (int e = 0; e < 4; e++) d[nt][e] = 0.f;
#pragma unroll
        for (int kk = 0; kk < 2; kk++) {
            // the inverse matrix flips the sign of the blocks that map Re <-> Im
            const uint32_t flip = (INV && ((kk == 0) == (nt >= 2))) ? 0x80008000u : 0u;
            const uint32_t bh0 = F.hi[kk][nt][0] ^ flip, bh1 = F.hi[kk][nt][1] ^ flip;
            const uint32_t bl0 = F.lo[kk][nt][0] ^ flip, bl1 = F.lo[kk][nt][1] ^ flip;
            mma_bf16(d[nt], al[kk], bh0, bh1);
            mma_bf16(d[nt], ah[kk], bl0, bl1);
            mma_bf16(d[nt], ah[kk], bh0, bh1);
        }
    }
    // d[nt][0..1]: row g, columns nt*8 + 2t + {0,1}; d[nt][2..3]: row g + 8
#pragma unroll
    for (int i = 0; i < 2; i++) {
        y[i][0] = make_float2(d[0][2 * i], d[2][2 * i]);
        y[i][1] = make_float2(d[0][2 * i + 1], d[2][2 * i + 1]);
        y[i][2] = make_float2(d[1][2 * i], d[3][2 * i]);
        y[i][3] = make_float2(d[1][2 * i + 1], d[3][2 * i + 1]);
    }
}

// forward (DIF) radix-16 pass of block size M: DFT then twiddle
template <class C, int M, int TOFF, int NTH, bool SMT>
__device__ __forceinline__ void fwd_pass_tc(float2* sm, const float2* tw, int tid) {
    constexpr int Q = M / 16, GROUPS = C::CS * (C::L / 16) / 16, NW = NTH / 32;
    const int lane = tid & 31, g = lane >> 2, t = lane & 3;
    TCFrag F;
    tc_matrix(F, lane);
    for (int grp = tid >> 5; grp < GROUPS; grp += NW) {
        float2* base[2];
        int n1s[2];
        float2 x[2][4], y[2][4];
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int it = grp * 16 + g + 8 * i;
            const int cs = it % C::CS, b = it / C::CS;
            n1s[i] = b % Q;
            base[i] = sm + cs * C::SP + (b / Q) * M + n1s[i];
#pragma unroll
            for (int j = 0; j < 4; j++) x[i][j] = base[i][tc_pos(t, j) * Q];
        }
        tc_dft<false>(x, y, F);
#pragma unroll
        for (int i = 0; i < 2; i++) {
            if (Q > 1) {
                const float4* w4 = reinterpret_cast<const float4*>(tw + TOFF + n1s[i] * 16 + 2 * t);
                const float4 w0 = tload<SMT>(w4), w1 = tload<SMT>(w4 + 4);   // k = 2t, 2t+1 and 2t+8, 2t+9
                y[i][0] = cmul(y[i][0], make_float2(w0.x, w0.y));
                y[i][1] = cmul(y[i][1], make_float2(w0.z, w0.w));
                y[i][2] = cmul(y[i][2], make_float2(w1.x, w1.y));
                y[i][3] = cmul(y[i][3], make_float2(w1.z, w1.w));
            }
#pragma unroll
            for (int j = 0; j < 4; j++) base[i][tc_pos(t, j) * Q] = y[i][j];
        }
    }
}

// inverse (DIT) radix-16 pass: conjugate twiddle then inverse DFT
template <class C, int M, int TOFF, int NTH, bool SMT>
__device__ __forceinline__ void inv_pass_tc(float2* sm, const float2* tw, int tid) {
    constexpr int Q = M / 16, GROUPS = C::CS * (C::L / 16) / 16, NW = NTH / 32;
    const int lane = tid & 31, g = lane >> 2, t = lane & 3;
    TCFrag F;
    tc_matrix(F, lane);
    for (int grp = tid >> 5; grp < GROUPS; grp += NW) {
        float2* base[2];
        float2 x[2][4], y[2][4];
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int it = grp * 16 + g + 8 * i;
            const int cs = it % C::CS, b = it / C::CS, n1 = b % Q;
            base[i] = sm + cs * C::SP + (b / Q) * M + n1;
#pragma unroll
            for (int j = 0; j < 4; j++) x[i][j] = base[i][tc_pos(t, j) * Q];
            if (Q > 1) {
                const float4* w4 = reinterpret_cast<const float4*>(tw + TOFF + n1 * 16 + 2 * t);
                const float4 w0 = tload<SMT>(w4), w1 = tload<SMT>(w4 + 4);
                x[i][0] = cmulc(x[i][0], make_float2(w0.x, w0.y));
                x[i][1] = cmulc(x[i][1], make_float2(w0.z, w0.w));
                x[i][2] = cmulc(x[i][2], make_float2(w1.x, w1.y));
                x[i][3] = cmulc(x[i][3], make_float2(w1.z, w1.w));
            }
        }
        tc_dft<true>(x, y, F);
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) base[i][tc_pos(t, j) * Q] = y[i][j];
    }
}

// last forward pass, derivative filter, first inverse pass (blocks of 16)
template <class C, int NTH, bool SMT>
__device__ __forceinline__ void mid_pass_tc(float2* sm, const float2* filt, int tid) {
    constexpr int GROUPS = C::CS * (C::L / 16) / 16, NW = NTH / 32;
    const int lane = tid & 31, g = lane >> 2, t = lane & 3;
    TCFrag F;
    tc_matrix(F, lane);
    for (int grp = tid >> 5; grp < GROUPS; grp += NW) {
        float2* base[2];
        int blks[2];
        float2 x[2][4], y[2][4];
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int it = grp * 16 + g + 8 * i;
            const int cs = it % C::CS;
            blks[i] = it / C::CS;
            base[i] = sm + cs * C::SP + blks[i] * 16;
#pragma unroll
            for (int j = 0; j < 4; j++) x[i][j] = base[i][tc_pos(t, j)];
        }
        tc_dft<false>(x, y, F);
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const float4* f4 = reinterpret_cast<const float4*>(filt + blks[i] * 16 + 2 * t);
            const float4 f0 = tload<SMT>(f4), f1 = tload<SMT>(f4 + 4);
            y[i][0] = cmul(y[i][0], make_float2(f0.x, f0.y));
            y[i][1] = cmul(y[i][1], make_float2(f0.z, f0.w));
            y[i][2] = cmul(y[i][2], make_float2(f1.x, f1.y));
            y[i][3] = cmul(y[i][3], make_float2(f1.z, f1.w));
        }
        tc_dft<true>(y, x, F);
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) base[i][tc_pos(t, j)] = x[i][j];
    }
}

// Two butterflies per thread and iteration: every load of both is issued
// before either is computed (the compiler cannot move a load above a shared
// store of the previous butterfly, so the one-at-a-time loop leaves a
// thread with a single butterfly's loads in flight).
template <class C, int R, int M>
__device__ __forceinline__ float2* pass_base(float2* sm, int it, int& n1) {
    constexpr int Q = M / R;
    const int cs = it % C::CS, b = it / C::CS;
    n1 = b % Q;
    return sm + cs * C::SP + (b / Q) * M + n1;
}

template <class C, int R, int M, int TOFF, int NTH, bool SMT, bool PRUNE>
__device__ __forceinline__ void fwd_pass_x2(float2* sm, const float2* tw, int tid, int lim) {
    constexpr int Q = M / R;
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it0 = tid; it0 < ITEMS; it0 += 2 * NTH) {
        float2 x[2][R];
        float2* base[2];
        int n1[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            base[u] = pass_base<C, R, M>(sm, it0 + u * NTH, n1[u]);
#pragma unroll
            for (int q = 0; q < R; q++)
                x[u][q] = (!PRUNE || n1[u] + q * Q < lim) ? base[u][q * Q] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            DFT<R, false>::run(x[u]);
            if (Q > 1) {
                float2 w[R];
                pass_twiddles<C, R, SMT>(tw + TOFF, n1[u], w);
#pragma unroll
                for (int k = 1; k < R; k++) x[u][k] = cmul(x[u][k], w[k]);
            }
#pragma unroll
            for (int k = 0; k < R; k++) base[u][k * Q] = x[u][k];
        }
    }
}

template <class C, int R, int M, int TOFF, int NTH, bool SMT, bool PRUNE>
__device__ __forceinline__ void inv_pass_x2(float2* sm, const float2* tw, int tid, int lo, int hi) {
    constexpr int Q = M / R;
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it0 = tid; it0 < ITEMS; it0 += 2 * NTH) {
        float2 x[2][R];
        float2* base[2];
        int n1[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            base[u] = pass_base<C, R, M>(sm, it0 + u * NTH, n1[u]);
#pragma unroll
            for (int k = 0; k < R; k++) x[u][k] = base[u][k * Q];
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (Q > 1) {
                float2 w[R];
                pass_twiddles<C, R, SMT>(tw + TOFF, n1[u], w);
#pragma unroll
                for (int k = 1; k < R; k++) x[u][k] = cmulc(x[u][k], w[k]);
            }
            DFT<R, true>::run(x[u]);
#pragma unroll
            for (int q = 0; q < R; q++)
                if (!PRUNE || (n1[u] + q * Q >= lo && n1[u] + q * Q < hi)) base[u][q * Q] = x[u][q];
        }
    }
}

// RM: rotation mask of mid_pass (position pairs rotated by the block index)
template <class C, int R, int NTH, bool SMT, int RM>
__device__ __forceinline__ void mid_pass_x2(float2* sm, const float2* filt, int tid) {
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it0 = tid; it0 < ITEMS; it0 += 2 * NTH) {
        float2 x[2][R];
        float2* base[2];
        int blk[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int it = it0 + u * NTH;
            const int cs = it % C::CS;
            blk[u] = it / C::CS;
            base[u] = sm + cs * C::SP + blk[u] * R;
            if constexpr (RM == 0) {
#pragma unroll
                for (int q = 0; q < R; q++) x[u][q] = base[u][q];
            } else {
                const int rot = 2 * (blk[u] & RM);
#pragma unroll
                for (int h = 0; h < R / 2; h++) {
                    const float4 v = *reinterpret_cast<const float4*>(base[u] + ((2 * h + rot) & (R - 1)));
                    x[u][2 * h] = make_float2(v.x, v.y);
                    x[u][2 * h + 1] = make_float2(v.z, v.w);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            DFT<R, false>::run(x[u]);
#pragma unroll
            for (int h = 0; h < R / 2; h++) {
                const float4 v = tload<SMT>(reinterpret_cast<const float4*>(filt + blk[u] * R) + h);
                x[u][2 * h] = cmul(x[u][2 * h], make_float2(v.x, v.y));
                x[u][2 * h + 1] = cmul(x[u][2 * h + 1], make_float2(v.z, v.w));
            }
            DFT<R, true>::run(x[u]);
            if constexpr (RM == 0) {
#pragma unroll
                for (int q = 0; q < R; q++) base[u][q] = x[u][q];
            } else {
                const int rot = 2 * (blk[u] & RM);
#pragma unroll
                for (int h = 0; h < R / 2; h++)
                    *reinterpret_cast<float4*>(base[u] + ((2 * h + rot) & (R - 1))) =
                        make_float4(x[u][2 * h].x, x[u][2 * h].y, x[u][2 * h + 1].x, x[u][2 * h + 1].y);
            }
        }
    }
}

template <class C, int R, int NTH>
__host__ __device__ constexpr bool use_x2() {
    return C::ILP && !C::TC && R <= 16 && (C::CS * (C::L / R)) % (2 * NTH) == 0;
}

// PRUNE (first pass, M = L): positions at or past `lim` hold the zero padding
// and are not loaded (nor stored by the gather)
template <class C, int R, int M, int TOFF, int NTH, bool SMT, bool PRUNE = false>
__device__ __forceinline__ void fwd_pass(float2* sm, const float2* tw, int tid, int lim = 0) {
    if constexpr (C::TC && R == 16) {
        fwd_pass_tc<C, M, TOFF, NTH, SMT>(sm, tw, tid);
        return;
    }
    if constexpr (use_x2<C, R, NTH>()) {
        fwd_pass_x2<C, R, M, TOFF, NTH, SMT, PRUNE>(sm, tw, tid, lim);
        return;
    }
    constexpr int Q = M / R;
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it = tid; it < ITEMS; it += NTH) {
        const int cs = it % C::CS, b = it / C::CS;
        const int blk = b / Q, n1 = b % Q;
        float2* base = sm + cs * C::SP + blk * M + n1;
        float2 x[R];
        if constexpr (R == 32) {
            static_assert(!C::CTW, "computed twiddles cover radix 2..16");
            // 32 values per thread: twiddles loaded pairwise after the butterfly
#pragma unroll
            for (int q = 0; q < R; q++)
                x[q] = (!PRUNE || n1 + q * Q < lim) ? base[q * Q] : make_float2(0.f, 0.f);
            DFT<R, false>::run(x);
            if (Q > 1) {
                const float4* t4 = reinterpret_cast<const float4*>(tw + TOFF + n1 * R);
#pragma unroll
                for (int h = 0; h < R / 2; h++) {
                    const float4 v = tload<SMT>(t4 + h);
                    if (h) x[2 * h] = cmul(x[2 * h], make_float2(v.x, v.y));
                    x[2 * h + 1] = cmul(x[2 * h + 1], make_float2(v.z, v.w));
                }
            }
        } else {
            float2 w[R];
            if (Q > 1) pass_twiddles<C, R, SMT>(tw + TOFF, n1, w);
#pragma unroll
            for (int q = 0; q < R; q++)
                x[q] = (!PRUNE || n1 + q * Q < lim) ? base[q * Q] : make_float2(0.f, 0.f);
            DFT<R, false>::run(x);
            if (Q > 1) {
#pragma unroll
                for (int k = 1; k < R; k++) x[k] = cmul(x[k], w[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < R; k++) base[k * Q] = x[k];
    }
}

// PRUNE (last pass, M = L): only positions in [lo, hi) -- the ones the
// epilogue reads -- are stored
template <class C, int R, int M, int TOFF, int NTH, bool SMT, bool PRUNE = false>
__device__ __forceinline__ void inv_pass(float2* sm, const float2* tw, int tid, int lo = 0, int hi = 0) {
    if constexpr (C::TC && R == 16) {
        inv_pass_tc<C, M, TOFF, NTH, SMT>(sm, tw, tid);
        return;
    }
    if constexpr (use_x2<C, R, NTH>()) {
        inv_pass_x2<C, R, M, TOFF, NTH, SMT, PRUNE>(sm, tw, tid, lo, hi);
        return;
    }
    constexpr int Q = M / R;
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it = tid; it < ITEMS; it += NTH) {
        const int cs = it % C::CS, b = it / C::CS;
        const int blk = b / Q, n1 = b % Q;
        float2* base = sm + cs * C::SP + blk * M + n1;
        float2 x[R];
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = base[k * Q];
        if (Q > 1) {
            if constexpr (R == 32) {
                static_assert(!C::CTW, "computed twiddles cover radix 2..16");
                const float4* t4 = reinterpret_cast<const float4*>(tw + TOFF + n1 * R);
#pragma unroll
                for (int h = 0; h < R / 2; h++) {
                    const float4 v = tload<SMT>(t4 + h);
                    if (h) x[2 * h] = cmulc(x[2 * h], make_float2(v.x, v.y));
                    x[2 * h + 1] = cmulc(x[2 * h + 1], make_float2(v.z, v.w));
                }
            } else {
                float2 w[R];
                pass_twiddles<C, R, SMT>(tw + TOFF, n1, w);
#pragma unroll
                for (int k = 1; k < R; k++) x[k] = cmulc(x[k], w[k]);
            }
        }
        DFT<R, true>::run(x);
#pragma unroll
        for (int q = 0; q < R; q++)
            if (!PRUNE || (n1 + q * Q >= lo && n1 + q * Q < hi)) base[q * Q] = x[q];
    }
}

// Rotation mask of the mid pass (see mid_pass): jobs of at most 4 strips with
// radix 4..16 (radix 32 would hold 16 rotated addresses); 16-byte accesses
// need an even strip pitch, which CS <= 4 gives (pad 16 / CS).
template <class C, int R>
__host__ __device__ constexpr int mid_rot_mask() {
    if (R < 4 || R > 16 || C::CS > 4 || (C::SP & 1)) return 0;
    return (8 / C::CS < R / 2 ? 8 / C::CS : R / 2) - 1;
}

// last forward pass (blocks of R contiguous positions), filter, first inverse pass
template <class C, int R, int NTH, bool SMT>
__device__ __forceinline__ void mid_pass(float2* sm, const float2* filt, int tid) {
    if constexpr (C::TC && R == 16) {
        mid_pass_tc<C, NTH, SMT>(sm, filt, tid);
        return;
    }
    if constexpr (use_x2<C, R, NTH>()) {
        mid_pass_x2<C, R, NTH, SMT, mid_rot_mask<C, R>()>(sm, filt, tid);
        return;
    }
    constexpr int ITEMS = C::CS * (C::L / R);
    for (int it = tid; it < ITEMS; it += NTH) {
        const int cs = it % C::CS, blk = it / C::CS;
        float2* base = sm + cs * C::SP + blk * R;
        // Registers 2h, 2h + 1 hold positions (2h + rot) mod R and the one
        // after it.  A circular shift of the input multiplies the spectrum by
        // a phase only; the filter leaves it and the inverse DFT turns it back
        // into the same shift, so each register is stored back where it came
        // from.  Blocks lie a multiple of 8 float2 apart and a quarter-warp
        // holds only CS strips, so without the shift its 16-byte accesses
        // meet in the same banks (2-way at CS = 4, 4-way at CS = 2).
        constexpr int RM = mid_rot_mask<C, R>();
        const int rot = 2 * (blk & RM);
        float2 x[R];
        if constexpr (RM == 0) {
#pragma unroll
            for (int q = 0; q < R; q++) x[q] = base[q];
        } else {
#pragma unroll
            for (int h = 0; h < R / 2; h++) {
                const float4 v = *reinterpret_cast<const float4*>(base + ((2 * h + rot) & (R - 1)));
                x[2 * h] = make_float2(v.x, v.y);
                x[2 * h + 1] = make_float2(v.z, v.w);
            }
        }
        DFT<R, false>::run(x);
#pragma unroll
        for (int h = 0; h < R / 2; h++) {
            const float4 v = tload<SMT>(reinterpret_cast<const float4*>(filt + blk * R) + h);
            x[2 * h] = cmul(x[2 * h], make_float2(v.x, v.y));
            x[2 * h + 1] = cmul(x[2 * h + 1], make_float2(v.z, v.w));
        }
        DFT<R, true>::run(x);
        if constexpr (RM == 0) {
#pragma unroll
            for (int q = 0; q < R; q++) base[q] = x[q];
        } else {
#pragma unroll
            for (int h = 0; h < R / 2; h++)
                *reinterpret_cast<float4*>(base + ((2 * h + rot) & (R - 1))) =
                    make_float4(x[2 * h].x, x[2 * h].y, x[2 * h + 1].x, x[2 * h + 1].y);
        }
    }
}

// PRUNE: the input is zero at and past z0 (not materialised) and only the
// output positions [lo, hi) are needed
template <class C, int NTH, int BAR, bool SMT, bool PRUNE = false>
__device__ __forceinline__ void convolve(float2* sm, const float2* tw, const float2* filt, int tid, int z0 = 0,
                                         int lo = 0, int hi = 0) {
    constexpr int M0 = C::L, M1 = C::M1, M2 = C::M2;
    constexpr int T0 = 0, T1 = C::T1, T2 = C::T2;
    if constexpr (C::NP == 2) {
        fwd_pass<C, C::R0, M0, T0, NTH, SMT, PRUNE>(sm, tw, tid, z0);
        group_sync<BAR, NTH>();
        mid_pass<C, C::R1, NTH, SMT>(sm, filt, tid);
        group_sync<BAR, NTH>();
        inv_pass<C, C::R0, M0, T0, NTH, SMT, PRUNE>(sm, tw, tid, lo, hi);
    } else if constexpr (C::NP == 3) {
        fwd_pass<C, C::R0, M0, T0, NTH, SMT, PRUNE>(sm, tw, tid, z0);
        group_sync<BAR, NTH>();
        fwd_pass<C, C::R1, M1, T1, NTH, SMT>(sm, tw, tid);
        group_sync<BAR, NTH>();
        mid_pass<C, C::R2, NTH, SMT>(sm, filt, tid);
        group_sync<BAR, NTH>();
        inv_pass<C, C::R1, M1, T1, NTH, SMT>(sm, tw, tid);
        group_sync<BAR, NTH>();
        inv_pass<C, C::R0, M0, T0, NTH, SMT, PRUNE>(sm, tw, tid, lo, hi);
    } else {
        fwd_pass<C, C::R0, M0, T0, NTH, SMT, PRUNE>(sm, tw, tid, z0);
        group_sync<BAR, NTH>();
        fwd_pass<C, C::R1, M1, T1, NTH, SMT>(sm, tw, tid);
        group_sync<BAR, NTH>();
        fwd_pass<C, C::R2, M2, T2, NTH, SMT>(sm, tw, tid);
        group_sync<BAR, NTH>();
        mid_pass<C, C::R3, NTH, SMT>(sm, filt, tid);
        group_sync<BAR, NTH>();
        inv_pass<C, C::R2, M2, T2, NTH, SMT>(sm, tw, tid);
        group_sync<BAR, NTH>();
        inv_pass<C, C::R1, M1, T1, NTH, SMT>(sm, tw, tid);
        group_sync<BAR, NTH>();
        inv_pass<C, C::R0, M0, T0, NTH, SMT, PRUNE>(sm, tw, tid, lo, hi);
    }
}

// reference operation order: dom = (band * T + mirror * R) * window
__device__ __forceinline__ float band_value(float raw, float mirror, float T, float R, float w) {
    return __fmul_rn(__fadd_rn(__fmul_rn(raw, T), __fmul_rn(mirror, R)), w);
}

// Field loads bypass L1 (the fields are streamed once per job), so that L1
// keeps the twiddle, filter and window tables every CTA of a bucket reads.
__device__ __forceinline__ float ldf(const float* p) {
    float v;
    asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float4 ldf4(const float* p) {   // p 16-byte aligned
    float4 v;
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p));
    return v;
}

// Source of the strip data of one domain in one stage.
struct Src {
    const float* a;   // p0 array (stale) or px, or the velocity field
    const float* b;   // py (p0 formed on the fly) or nullptr
    int pitch;
    __device__ __forceinline__ float at(long long e) const {
        return b ? __fadd_rn(ldf(a + e), ldf(b + e)) : ldf(a + e);
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
        u = ldf4(p + i);
    } else {
        u.x = ldf(p + i);
        if (i + 1 < n) u.y = ldf(p + i + 1);
        if (i + 2 < n) u.z = ldf(p + i + 2);
    }
    return u;
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}

// Carry the fields of a non-updated axis through the stage: the derivative
// array keeps its zero content, so the RK update returns the stage-start value.
template <int NTH>
__device__ void copy_axis(const StageArgs& A, const DevDomain& D, bool ydir, int tid) {
    if (!ydir) {
        for (int k = tid; k < D.ny * (D.nx + 1); k += NTH) {
            const int r = k / (D.nx + 1), i = k - r * (D.nx + 1);
            const long long e = D.o_vx + (long long)r * D.pitch_vx + i;
            float v = A.prev[e];
            if (A.last && D.att_xv >= 0) v = __fmul_rn(v, A.att[D.att_xv + i]);
            A.out[e] = v;
        }
        for (int k = tid; k < D.ny * D.nx; k += NTH) {
            const int r = k / D.nx, i = k - r * D.nx;
            const long long e = D.o_px + (long long)r * D.pitch_p + i;
            A.out[e] = A.prev[e];
        }
    } else {
        for (int k = tid; k < (D.ny + 1) * D.nx; k += NTH) {
            const int r = k / D.nx, i = k - r * D.nx;
            const long long e = D.o_vy + (long long)r * D.pitch_vy + i;
            float v = A.prev[e];
            if (A.last && D.att_yv >= 0) v = __fmul_rn(v, A.att[D.att_yv + r]);
            A.out[e] = v;
        }
        for (int k = tid; k < D.ny * D.nx; k += NTH) {
            const int r = k / D.nx, i = k - r * D.nx;
            const long long e = D.o_py + (long long)r * D.pitch_p + i;
            A.out[e] = A.prev[e];
        }
    }
}

// ---- step 1: strips + bands + padding of one job into `sm` (NTH threads)
// TWO: the strip's p0 is formed as px + py (else one field: velocity or stale p0)
// Four positions of a row pair (strips 2cs, 2cs + 1 interleaved as one
// complex strip) as two 16-byte shared accesses; d must be 16-byte aligned.
__device__ __forceinline__ void store_pairs(float2* d, float4 u, float4 v) {
    float4* d4 = reinterpret_cast<float4*>(d);
    d4[0] = make_float4(u.x, v.x, u.y, v.y);
    d4[1] = make_float4(u.z, v.z, u.w, v.w);
}
__device__ __forceinline__ void load_pairs(const float2* s, float2 (&d)[4]) {
    const float4 a = reinterpret_cast<const float4*>(s)[0], b = reinterpret_cast<const float4*>(s)[1];
    d[0] = make_float2(a.x, a.y);
    d[1] = make_float2(a.z, a.w);
    d[2] = make_float2(b.x, b.y);
    d[3] = make_float2(b.z, b.w);
}

template <class C, int NTH, bool ZERO, bool TWO>
__device__ __forceinline__ void gather_k(float2* sm, const StageArgs& A, const DevJob& job, const DevDomain& dom,
                                         bool first, const Src& S, int tid) {
    constexpr int CS = C::CS, SP = C::SP, L = C::L, S2 = 2 * CS;
    constexpr int NW = NTH / 32;
    constexpr int WPP = NW >= CS ? NW / CS : 1;   // warps per strip pair
    constexpr int PST = NW / WPP;                 // strip pairs in flight
    float* smf = reinterpret_cast<float*>(sm);
    const int warp = tid >> 5, lane = tid & 31;
    const bool vel = job.kind & JK_VEL;
    const bool ydir = job.kind & JK_Y;
    const int W = job.W;
    const int n = (ydir ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int count = job.count;
    if (!ydir) {
        // row pairs (2cs, 2cs+1), 16-byte loads, four chunks per lane in flight
        const int chunks = (n + 3) >> 2;
        const bool pair16 = (SP % 2 == 0) && !(W & 1);   // 16-byte aligned pairs in shared memory
        if (WPP == 1 && chunks <= 16) {
            // short rows (the PML-normal strips): a half-warp per row pair
            const int l16 = lane & 15, i = l16 << 2;
#pragma unroll 2
            for (int cs = 2 * warp + (lane >> 4); cs < CS; cs += 2 * NW) {
                if (l16 >= chunks) continue;
                const int s0 = 2 * cs;
                const float* a0 = S.a + (long long)(job.first + s0) * S.pitch;
                const float* b0 = TWO ? S.b + (long long)(job.first + s0) * S.pitch : nullptr;
                float4 u = make_float4(0.f, 0.f, 0.f, 0.f), v = u;
                if (s0 < count) u = TWO ? add4(ldf4(a0 + i), ldf4(b0 + i)) : ldf4(a0 + i);
                if (s0 + 1 < count) v = TWO ? add4(ldf4(a0 + S.pitch + i), ldf4(b0 + S.pitch + i)) : ldf4(a0 + S.pitch + i);
                float2* d = sm + cs * SP + W + i;
                if (pair16 && i + 4 <= n) {
                    store_pairs(d, u, v);
                } else {
                    d[0] = make_float2(u.x, v.x);
                    if (i + 1 < n) d[1] = make_float2(u.y, v.y);
                    if (i + 2 < n) d[2] = make_float2(u.z, v.z);
                    if (i + 3 < n) d[3] = make_float2(u.w, v.w);
                }
            }
        } else
        for (int cs = warp / WPP; cs < CS; cs += PST) {
            const int s0 = 2 * cs;
            const float* a0 = S.a + (long long)(job.first + s0) * S.pitch;
            const float* b0 = TWO ? S.b + (long long)(job.first + s0) * S.pitch : nullptr;
            const bool h0 = s0 < count, h1 = s0 + 1 < count;
            for (int c0 = (warp % WPP) * 32 + lane; c0 < chunks; c0 += 2 * WPP * 32) {
                float4 u[4], v[4];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int c = c0 + q * WPP * 32, i = c << 2;
                    u[q] = v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (c < chunks) {
                        // whole 16-byte quads: every row is padded past its last quad
                        if (h0) u[q] = TWO ? add4(ldf4(a0 + i), ldf4(b0 + i)) : ldf4(a0 + i);
                        if (h1) v[q] = TWO ? add4(ldf4(a0 + S.pitch + i), ldf4(b0 + S.pitch + i)) : ldf4(a0 + S.pitch + i);
                    }
                }
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int c = c0 + q * WPP * 32, i = c << 2;
                    if (c < chunks) {
                        float2* d = sm + cs * SP + W + i;
                        if (pair16 && i + 4 <= n) {
                            store_pairs(d, u[q], v[q]);
                        } else {
                            d[0] = make_float2(u[q].x, v[q].x);
                            if (i + 1 < n) d[1] = make_float2(u[q].y, v[q].y);
                            if (i + 2 < n) d[2] = make_float2(u[q].z, v[q].z);
                            if (i + 3 < n) d[3] = make_float2(u[q].w, v[q].w);
                        }
                    }
                }
            }
        }
    } else if (S2 % 4 == 0 && count == S2 && (job.first & 3) == 0) {
        // columns, four adjacent strips per 16-byte load (rows are 128-byte
        // aligned and the job starts on a multiple of four columns); four
        // quads per thread in flight
        constexpr int G = S2 / 4;
        const int total = G * n;
        for (int f0 = tid; f0 < total; f0 += 4 * NTH) {
            float4 u[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                if (f < total) {
                    const int g = f % G, i = f / G;
                    const float* a = S.a + (long long)i * S.pitch + job.first + 4 * g;
                    u[q] = TWO ? add4(ldf4(a), ldf4(S.b + (a - S.a))) : ldf4(a);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                if (f < total) {
                    const int g = f % G, i = f / G;
                    sm[2 * g * SP + W + i] = make_float2(u[q].x, u[q].y);
                    sm[(2 * g + 1) * SP + W + i] = make_float2(u[q].z, u[q].w);
                }
            }
        }
    } else {
        // columns: consecutive threads read consecutive columns of one row,
        // four elements per thread in flight
        const int total = S2 * n;
        for (int f0 = tid; f0 < total; f0 += 4 * NTH) {
            float val[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                val[q] = 0.f;
                if (f < total) {
                    const int s = f % S2, i = f / S2;
                    if (s < count) {
                        const long long el = (long long)i * S.pitch + job.first + s;
                        val[q] = TWO ? __fadd_rn(ldf(S.a + el), ldf(S.b + el)) : ldf(S.a + el);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                if (f < total) {
                    const int s = f % S2, i = f / S2;
                    smf[2 * ((s >> 1) * SP + W + i) + (s & 1)] = val[q];
                }
            }
        }
    }
    // interface bands: one warp per strip, lanes along the band
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
    // zero padding [2W+n, L) of every complex strip (a pruned first pass does
    // not read it)
    if constexpr (ZERO) {
        const int z0 = 2 * W + n;
        for (int cs = warp; cs < CS; cs += NW)
            for (int p = z0 + lane; p < L; p += 32) sm[cs * SP + p] = make_float2(0.f, 0.f);
    }
}

template <class C, int NTH, bool ZERO = true>
__device__ __forceinline__ void gather(float2* sm, const StageArgs& A, const DevJob& job, const DevDomain& dom,
                                       bool first, int tid) {
    const Src S = strip_source(A, dom, job.kind & JK_VEL, job.kind & JK_Y, first);
    if (S.b) gather_k<C, NTH, ZERO, true>(sm, A, job, dom, first, S, tid);
    else gather_k<C, NTH, ZERO, false>(sm, A, job, dom, first, S, tid);
}

// ---- step 5: slice, RK update, (sixth stage) PML on vx / vy
// RK update of one value in the reference's operation order
// (kernel/Solver.cpp:174-181): v0 - (dt*a_k) * (L / rho) and p0 - (dt*a_k) * ((L*rho)*c^2)
__device__ __forceinline__ float div_rho(float d, float rho, float rinv) {
    // d / rho correctly rounded from the correctly rounded reciprocal rinv:
    // q = d * rinv, exact residual r = d - q * rho (FMA), q + r * rinv
    // (Markstein's division correction, "IA-64 and Elementary Functions",
    // 2000, section 8); rho is a finite normal density, d a field derivative
    const float q = __fmul_rn(d, rinv);
    const float r = __fmaf_rn(-q, rho, d);
    return __fmaf_rn(r, rinv, q);
}

__device__ __forceinline__ float rk_update(float prev, float d, bool vel, float cdt, float rho, float c2, float rinv) {
    return vel ? __fsub_rn(prev, __fmul_rn(cdt, __fmul_rn(__fmul_rn(d, rho), c2)))
               : __fsub_rn(prev, __fmul_rn(cdt, div_rho(d, rho, rinv)));
}

template <class C, int NTH, bool VEL, bool ATT>
__device__ __forceinline__ void epilogue_k(const float2* sm, const StageArgs& A, const DevJob& job, const DevDomain& dom,
                                           int tid) {
    constexpr int CS = C::CS, SP = C::SP, S2 = 2 * CS;
    constexpr int NW = NTH / 32;
    constexpr int WPP = NW >= CS ? NW / CS : 1;
    constexpr int PST = NW / WPP;
    const float* smf = reinterpret_cast<const float*>(sm);
    const float* __restrict__ prev = A.prev;
    float* __restrict__ out = A.out;
    const int warp = tid >> 5, lane = tid & 31;
    constexpr bool vel = VEL;
    const bool ydir = job.kind & JK_Y;
    const int W = job.W;
    const int n = (ydir ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int count = job.count;
    const float cdt = A.doms[job.dom].cdt[A.stage];
    const float rho = dom.rho;
    const float c2 = dom.c2;
    const float rinv = __frcp_rn(rho);
    const int nout = vel ? n - 1 : n + 1;   // cells (vel) or faces (pressure)
    long long fo;
    int fp, ao;
    if (!vel) { fo = ydir ? dom.o_vy : dom.o_vx; fp = ydir ? dom.pitch_vy : dom.pitch_vx; ao = ydir ? dom.att_yv : dom.att_xv; }
    else { fo = ydir ? dom.o_py : dom.o_px; fp = dom.pitch_p; ao = -1; }
    constexpr bool att = ATT;   // PML multiply of vx / vy at the sixth stage
    if (!ydir) {
        // rows: four consecutive outputs per lane (16-byte loads / stores), two chunks in flight
        const int chunks = (nout + 3) >> 2;
        const bool pair16 = (SP % 2 == 0) && !(W & 1);   // 16-byte aligned pairs in shared memory
        if (WPP == 1 && chunks <= 16) {
            // short rows (the PML-normal strips): a half-warp per row pair
            const int l16 = lane & 15, i = l16 << 2;
#pragma unroll 2
            for (int cs = 2 * warp + (lane >> 4); cs < CS; cs += 2 * NW) {
                if (l16 >= chunks || 2 * cs >= count) continue;
                const long long r0 = fo + (long long)(job.first + 2 * cs) * fp;
                const bool h1 = 2 * cs + 1 < count;
                const float4 p0v = ldf4(prev + r0 + i);   // whole quads: rows are padded
                const float4 p1v = h1 ? ldf4(prev + r0 + fp + i) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float2* srow = sm + cs * SP + W;
                float2 d[4];
                if (pair16 && i + 4 <= nout) {
                    load_pairs(srow + i, d);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; e++) d[e] = (i + e < nout) ? srow[i + e] : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (h == 1 && !h1) break;
                    const float4 pv = h ? p1v : p0v;
                    float v[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        v[e] = rk_update(v[e], h ? d[e].y : d[e].x, vel, cdt, rho, c2, rinv);
                        if (att && i + e < nout) v[e] = __fmul_rn(v[e], A.att[ao + i + e]);
                    }
                    float* o = out + r0 + (h ? fp : 0) + i;
                    if (i + 4 <= nout) {
                        *reinterpret_cast<float4*>(o) = make_float4(v[0], v[1], v[2], v[3]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; e++)
                            if (i + e < nout) o[e] = v[e];
                    }
                }
            }
        } else
        for (int cs = warp / WPP; cs < CS; cs += PST) {
            const float2* srow = sm + cs * SP + W;
            const long long r0 = fo + (long long)(job.first + 2 * cs) * fp;
            const bool h1 = 2 * cs + 1 < count;
            if (2 * cs >= count) continue;
            for (int c0 = (warp % WPP) * 32 + lane; c0 < chunks; c0 += 2 * WPP * 32) {
                float4 p[2][2];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int i = (c0 + q * WPP * 32) << 2;
                    p[q][0] = p[q][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (i < nout) {
                        // whole quads: rows are padded past their last quad
                        p[q][0] = ldf4(prev + r0 + i);
                        if (h1) p[q][1] = ldf4(prev + r0 + fp + i);
                    }
                }
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int i = (c0 + q * WPP * 32) << 2;
                    if (i >= nout) continue;
                    float2 d[4];
                    if (pair16 && i + 4 <= nout) {
                        load_pairs(srow + i, d);
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; e++) d[e] = (i + e < nout) ? srow[i + e] : make_float2(0.f, 0.f);
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (h == 1 && !h1) break;
                        float v[4] = {p[q][h].x, p[q][h].y, p[q][h].z, p[q][h].w};
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            v[e] = rk_update(v[e], h ? d[e].y : d[e].x, vel, cdt, rho, c2, rinv);
                            if (att && i + e < nout) v[e] = __fmul_rn(v[e], A.att[ao + i + e]);
                        }
                        float* o = out + r0 + (h ? fp : 0) + i;
                        if (i + 4 <= nout) {
                            *reinterpret_cast<float4*>(o) = make_float4(v[0], v[1], v[2], v[3]);
                        } else {
#pragma unroll
                            for (int e = 0; e < 4; e++)
                                if (i + e < nout) o[e] = v[e];
                        }
                    }
                }
            }
        }
    } else if (S2 % 4 == 0 && count == S2 && (job.first & 3) == 0) {
        // columns, four adjacent strips per 16-byte load / store, four quads in flight
        constexpr int G = S2 / 4;
        const int total = G * nout;
        for (int f0 = tid; f0 < total; f0 += 4 * NTH) {
            float4 pv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                if (f < total) {
                    const int g = f % G, i = f / G;
                    pv[q] = ldf4(prev + fo + (long long)i * fp + job.first + 4 * g);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                if (f >= total) continue;
                const int g = f % G, i = f / G;
                const float2 d0 = sm[2 * g * SP + W + i], d1 = sm[(2 * g + 1) * SP + W + i];
                float v[4] = {rk_update(pv[q].x, d0.x, vel, cdt, rho, c2, rinv), rk_update(pv[q].y, d0.y, vel, cdt, rho, c2, rinv),
                              rk_update(pv[q].z, d1.x, vel, cdt, rho, c2, rinv), rk_update(pv[q].w, d1.y, vel, cdt, rho, c2, rinv)};
                if (att) {
                    const float a = A.att[ao + i];
#pragma unroll
                    for (int e = 0; e < 4; e++) v[e] = __fmul_rn(v[e], a);
                }
                *reinterpret_cast<float4*>(out + fo + (long long)i * fp + job.first + 4 * g) =
                    make_float4(v[0], v[1], v[2], v[3]);
            }
        }
    } else {
        // columns: consecutive threads on consecutive columns, four values in flight
        const int total = S2 * nout;
        for (int f0 = tid; f0 < total; f0 += 4 * NTH) {
            float pv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                const int s = f % S2, i = f / S2;
                pv[q] = (f < total && s < count) ? ldf(prev + fo + (long long)i * fp + job.first + s) : 0.f;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int f = f0 + q * NTH;
                const int s = f % S2, i = f / S2;
                if (f >= total || s >= count) continue;
                const float dv = smf[2 * ((s >> 1) * SP + W + i) + (s & 1)];
                float v = rk_update(pv[q], dv, vel, cdt, rho, c2, rinv);
                if (att) v = __fmul_rn(v, A.att[ao + i]);
                out[fo + (long long)i * fp + job.first + s] = v;
            }
        }
    }
}

// the update arithmetic differs between velocity and pressure derivatives:
// one instantiation each, chosen once per job
template <class C, int NTH>
__device__ __forceinline__ void epilogue(const float2* sm, const StageArgs& A, const DevJob& job, const DevDomain& dom,
                                         int tid) {
    const int ao = (job.kind & JK_Y) ? dom.att_yv : dom.att_xv;
    if (job.kind & JK_VEL) epilogue_k<C, NTH, true, false>(sm, A, job, dom, tid);
    else if (A.last && ao >= 0) epilogue_k<C, NTH, false, true>(sm, A, job, dom, tid);
    else epilogue_k<C, NTH, false, false>(sm, A, job, dom, tid);
}

// ---------------------------------------------------------------- plain form
template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_kernel(StageArgs A) {
    extern __shared__ __align__(16) float2 sm[];
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    if (job.kind & JK_COPY) {
        copy_axis<C::NT>(A, dom, job.kind & JK_Y, threadIdx.x);
        return;
    }
    const bool first = A.first_step[dom.scene] != 0;
    constexpr bool PRUNE = !C::TC;   // the tensor-core passes read the padding
    gather<C, C::NT, !PRUNE>(sm, A, job, dom, first, threadIdx.x);
    __syncthreads();
    const bool vel = job.kind & JK_VEL;
    const int n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int nout = vel ? n - 1 : n + 1;
    convolve<C, C::NT, 0, false, PRUNE>(sm, A.tw, A.filt + job.dtab, threadIdx.x, 2 * job.W + n, job.W,
                                         job.W + nout);
    __syncthreads();
    epilogue<C, C::NT>(sm, A, job, dom, threadIdx.x);
}

// The plain stage kernel as a persistent loop over a job table whose length
// is read from device memory (serving loop): resident CTAs take jobs from
// *counter; all-zero entries (free table ranges: length 0, no copy flag) and
// jobs of scenes that have taken all their steps are skipped.
template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_kernel_dev(const __grid_constant__ StageArgs A, const int* count,
                                                                  int* counter) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ int s_job;
    const int n = *count;
    for (;;) {
        if (threadIdx.x == 0) s_job = atomicAdd(counter, 1);
        __syncthreads();
        const int j = s_job;
        if (j >= n) break;   // the same value for the whole CTA
        const DevJob job = A.jobs[j];
        const DevDomain dom = A.doms[job.dom];
        const bool live = !A.scene_limit || A.scene_step[dom.scene] < A.scene_limit[dom.scene];
        if (!live || (job.L == 0 && !(job.kind & JK_COPY))) {
        } else if (job.kind & JK_COPY) {
            copy_axis<C::NT>(A, dom, job.kind & JK_Y, threadIdx.x);
        } else {
            const bool first = A.first_step[dom.scene] != 0;
            gather<C, C::NT, false>(sm, A, job, dom, first, threadIdx.x);
            __syncthreads();
            const bool vel = job.kind & JK_VEL;
            const int nn = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
            const int nout = vel ? nn - 1 : nn + 1;
            convolve<C, C::NT, 0, false, true>(sm, A.tw, A.filt + job.dtab, threadIdx.x, 2 * job.W + nn, job.W,
                                               job.W + nout);
            __syncthreads();
            epilogue<C, C::NT>(sm, A, job, dom, threadIdx.x);
        }
        __syncthreads();   // shared memory and s_job are reused by the next job
    }
}

// ---------------------------------------------------------------- persistent form
// named barriers: 1,2 buffer full; 3,4 buffer transformed; 5 FFT warps; 6 memory warps
template <class C>
__global__ void __launch_bounds__(C::NT + C::NTP, 1) stage_ws(StageArgs A, int n_jobs) {
    constexpr int NTC = C::NT, NTP = C::NTP, ALL = C::NT + C::NTP;
    extern __shared__ __align__(16) float2 sm[];
    float2* tws = sm + 2 * C::BUF;
    float2* flt = tws + C::TWN;
    const int tid = threadIdx.x;
    // stage the twiddle tables and both derivative filters once
    {
        const float4* s4 = reinterpret_cast<const float4*>(A.tw);
        float4* d4 = reinterpret_cast<float4*>(tws);
        for (int i = tid; i < C::TWN / 2; i += ALL) d4[i] = __ldg(s4 + i);
        const float4* p4 = reinterpret_cast<const float4*>(A.filt_p);
        const float4* v4 = reinterpret_cast<const float4*>(A.filt_v);
        float4* f4 = reinterpret_cast<float4*>(flt);
        for (int i = tid; i < C::L / 2; i += ALL) {
            f4[i] = __ldg(p4 + i);
            f4[C::L / 2 + i] = __ldg(v4 + i);
        }
    }
    __syncthreads();
    const int stride = gridDim.x;
    const int mine = (int)blockIdx.x < n_jobs ? (n_jobs - 1 - (int)blockIdx.x) / stride + 1 : 0;
    if (tid < NTC) {
        // FFT warps
        for (int k = 0; k < mine; k++) {
            const int b = k & 1;
            const int kind = A.jobs[blockIdx.x + k * stride].kind;
            bar_sync(1 + b, ALL);
            if (!(kind & JK_COPY))
                convolve<C, NTC, 5, true>(sm + b * C::BUF, tws, flt + ((kind & JK_VEL) ? C::L : 0), tid);
            bar_arrive(3 + b, ALL);
        }
    } else {
        // memory warps: gather job k while the FFT warps transform job k-1,
        // then write back job k-1
        const int ptid = tid - NTC;
        for (int k = 0; k <= mine; k++) {
            if (k < mine) {
                const int b = k & 1;
                const DevJob job = A.jobs[blockIdx.x + k * stride];
                const DevDomain dom = A.doms[job.dom];
                if (!(job.kind & JK_COPY)) gather<C, NTP>(sm + b * C::BUF, A, job, dom, A.first_step[dom.scene] != 0, ptid);
                bar_arrive(1 + b, ALL);
            }
            if (k >= 1) {
                const int b = (k - 1) & 1;
                const DevJob job = A.jobs[blockIdx.x + (k - 1) * stride];
                bar_sync(3 + b, ALL);
                const DevDomain dom = A.doms[job.dom];
                if (job.kind & JK_COPY) copy_axis<NTP>(A, dom, job.kind & JK_Y, ptid);
                else epilogue<C, NTP>(sm + b * C::BUF, A, job, dom, ptid);
                group_sync<6, NTP>();   // buffer b is gathered again at iteration k+1
            }
        }
    }
}

// ---------------------------------------------------------------- pipelined form
// Persistent CTAs walk the job list; the strips, interface bands and
// stage-start values of job k+2 are copied global -> shared with cp.async
// (no registers held, every copy of a job in flight at once) while job k is
// transformed.  Each thread waits only for its own copy groups
// (cp.async.wait_group) and a CTA barrier then publishes them, so there is no
// spin wait.  Shared memory: the FFT buffer, then two staging slots of
//   A[S2][rc] / B[S2][rc] / P[S2][rc]   (rows of x jobs; [rc][S2] for y jobs)
//   bands[2 sides][2 fields][S2][32]
// where A = px (or vx, vy, stale p0), B = py (p0 formed as A + B), P = the
// stage-start values of the updated field.
constexpr int PIPE_WB = 32;   // band slots per strip (windows are at most 32 wide)

__device__ __forceinline__ void cp16(float* dst, const float* src) {   // both 16-byte aligned
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp4(float* dst, const float* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__host__ __device__ constexpr int pipe_slot_floats(int S2, int rc) { return 3 * S2 * rc + 4 * S2 * PIPE_WB; }

// geometry of one job shared by staging, blending and the epilogue
struct PipeJob {
    bool vel, ydir, vec;   // vec: y job on four-aligned full columns (16-byte copies)
    int n, nout, W, count;
    long long fo;          // offset of the updated field in a state set
    int fp, ao;            // its pitch; attenuation offset (-1 = none)
    Src S;
};

template <int S2>
__device__ __forceinline__ PipeJob pipe_job(const StageArgs& A, const DevJob& job, const DevDomain& dom, bool first) {
    PipeJob g;
    g.vel = job.kind & JK_VEL;
    g.ydir = job.kind & JK_Y;
    g.n = (g.ydir ? dom.ny : dom.nx) + (g.vel ? 1 : 0);
    g.nout = g.vel ? g.n - 1 : g.n + 1;
    g.W = job.W;
    g.count = job.count;
    g.vec = g.ydir && S2 % 4 == 0 && job.count == S2 && (job.first & 3) == 0;
    if (!g.vel) {
        g.fo = g.ydir ? dom.o_vy : dom.o_vx;
        g.fp = g.ydir ? dom.pitch_vy : dom.pitch_vx;
        g.ao = g.ydir ? dom.att_yv : dom.att_xv;
    } else {
        g.fo = g.ydir ? dom.o_py : dom.o_px;
        g.fp = dom.pitch_p;
        g.ao = -1;
    }
    g.S = strip_source(A, dom, g.vel, g.ydir, first);
    return g;
}

// issue every copy of one job into `slot` (all NTH threads)
template <class C, int NTH>
__device__ __forceinline__ void pipe_stage_in(float* slot, const StageArgs& A, const DevJob& job, int rc, int tid) {
    constexpr int S2 = 2 * C::CS;
    const DevDomain dom = A.doms[job.dom];
    const bool first = A.first_step[dom.scene] != 0;
    const PipeJob g = pipe_job<S2>(A, job, dom, first);
    float* sa = slot;
    float* sb = slot + S2 * rc;
    float* sp = slot + 2 * S2 * rc;
    float* sband = slot + 3 * S2 * rc;
    const float* P = A.prev + g.fo;
    const Src& S = g.S;
    const int nf = S.b ? 2 : 1;
    if (!g.ydir) {
        // rows: whole 16-byte quads (the last one reads into the row's padding)
        const int qa = (g.n + 3) >> 2, qp = (g.nout + 3) >> 2;
        const int per = nf * qa + qp;
        for (int k = tid; k < g.count * per; k += NTH) {
            const int s = k / per, q = k - s * per;
            const long long row = job.first + s;
            if (q < qa) cp16(sa + s * rc + 4 * q, S.a + row * S.pitch + 4 * q);
            else if (q < nf * qa) cp16(sb + s * rc + 4 * (q - qa), S.b + row * S.pitch + 4 * (q - qa));
            else cp16(sp + s * rc + 4 * (q - nf * qa), P + row * g.fp + 4 * (q - nf * qa));
        }
    } else if (g.vec) {
        constexpr int G = S2 / 4;
        const int tin = g.n * G;
        for (int k = tid; k < nf * tin + g.nout * G; k += NTH) {
            if (k < nf * tin) {
                const int f = k >= tin, r = k - f * tin;
                const int q = r % G, i = r / G;
                cp16((f ? sb : sa) + i * S2 + 4 * q, (f ? S.b : S.a) + (long long)i * S.pitch + job.first + 4 * q);
            } else {
                const int r = k - nf * tin, q = r % G, i = r / G;
                cp16(sp + i * S2 + 4 * q, P + (long long)i * g.fp + job.first + 4 * q);
            }
        }
    } else {
        // columns of a ragged or unaligned job: 4-byte copies
        const int tin = g.n * g.count;
        for (int k = tid; k < nf * tin + g.nout * g.count; k += NTH) {
            if (k < nf * tin) {
                const int f = k >= tin, r = k - f * tin;
                const int s = r % g.count, i = r / g.count;
                cp4((f ? sb : sa) + i * S2 + s, (f ? S.b : S.a) + (long long)i * S.pitch + job.first + s);
            } else {
                const int r = k - nf * tin, s = r % g.count, i = r / g.count;
                cp4(sp + i * S2 + s, P + (long long)i * g.fp + job.first + s);
            }
        }
    }
    // interface bands of the neighbours: the W values next to the interface
    const int W = g.W;
    for (int d = 0; d < 2; d++) {
        const int nb = d ? job.d2 : job.d1;
        if (nb < 0) continue;
        const DevDomain D = A.doms[nb];
        const Src T = strip_source(A, D, g.vel, g.ydir, first);
        const int nn = (g.ydir ? D.ny : D.nx) + (g.vel ? 1 : 0);
        const int e0 = d ? (g.vel ? 1 : 0) : (g.vel ? nn - W - 1 : nn - W);
        const int o = d ? job.o2 : job.o1;
        // pressure bands keep two fields (px, py); a neighbour that supplies
        // one (stale p0) gets a zero second field, so the blend adds exactly
        const int tf = g.count * W;
        for (int k = tid; k < (g.vel ? 1 : 2) * tf; k += NTH) {
            const int f = k >= tf, r = k - f * tf;
            const int s = r / W, j = r - s * W;
            float* dst = sband + ((2 * d + f) * S2 + s) * PIPE_WB + j;
            if (f && !T.b) {
                *dst = 0.f;
                continue;
            }
            const float* src = f ? T.b : T.a;
            const long long e = g.ydir ? (long long)(e0 + j) * T.pitch + o + s : (long long)(o + s) * T.pitch + e0 + j;
            cp4(dst, src + e);
        }
    }
}

// staged own strip value s at index i (p0 formed as A + B)
template <int S2>
__device__ __forceinline__ float pipe_own(const float* sa, const float* sb, bool two, bool ydir, int rc, int s, int i) {
    const int e = ydir ? i * S2 + s : s * rc + i;
    return two ? __fadd_rn(sa[e], sb[e]) : sa[e];
}

// staging slot -> complex strips of the FFT buffer (bands blended, zero padded)
template <class C, int NTH>
__device__ __forceinline__ void pipe_blend(float2* sm, const float* slot, const StageArgs& A, const DevJob& job,
                                           const PipeJob& g, int rc, int tid) {
    constexpr int CS = C::CS, SP = C::SP, L = C::L, S2 = 2 * CS;
    const float* sa = slot;
    const float* sb = slot + S2 * rc;
    const float* sband = slot + 3 * S2 * rc;
    const bool two = g.S.b != nullptr;
    const int W = g.W, n = g.n;
    const float* wl = A.win + job.wtab;          // window.head(W)
    const float* wr = A.win + job.wtab + W + 1;  // window.tail(W)
    for (int it = tid; it < CS * L; it += NTH) {
        // x jobs: consecutive threads along a strip; y jobs: along the strip pairs
        const int cs = g.ydir ? it % CS : it / L;
        const int p = g.ydir ? it / CS : it % L;
        float v[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int s = 2 * cs + h;
            float val = 0.f;
            if (s < g.count) {
                if (p < W) {
                    if (job.d1 >= 0) {
                        const float* b = sband + (0 * S2 + s) * PIPE_WB + p;
                        const float raw = g.vel ? b[0] : __fadd_rn(b[0], b[S2 * PIPE_WB]);
                        const int m = g.vel ? W - p : W - 1 - p;
                        val = band_value(raw, pipe_own<S2>(sa, sb, two, g.ydir, rc, s, m), job.T1, job.R1, __ldg(wl + p));
                    }
                } else if (p < W + n) {
                    val = pipe_own<S2>(sa, sb, two, g.ydir, rc, s, p - W);
                } else if (p < 2 * W + n) {
                    const int jj = p - W - n;
                    if (job.d2 >= 0) {
                        const float* b = sband + (2 * S2 + s) * PIPE_WB + jj;
                        const float raw = g.vel ? b[0] : __fadd_rn(b[0], b[S2 * PIPE_WB]);
                        const int m = g.vel ? n - 2 - jj : n - 1 - jj;
                        val = band_value(raw, pipe_own<S2>(sa, sb, two, g.ydir, rc, s, m), job.T2, job.R2, __ldg(wr + jj));
                    }
                }
            }
            v[h] = val;
        }
        sm[cs * SP + p] = make_float2(v[0], v[1]);
    }
}

// slice, RK update against the staged stage-start values sp, store
template <class C, int NTH>
__device__ __forceinline__ void pipe_epilogue(const float2* sm, const float* sp, const StageArgs& A, const DevJob& job,
                                              const DevDomain& dom, const PipeJob& g, int rc, int tid) {
    constexpr int CS = C::CS, SP = C::SP, S2 = 2 * CS;
    float* __restrict__ out = A.out;
    const float cdt = A.doms[job.dom].cdt[A.stage];
    const float rho = dom.rho, c2 = dom.c2, rinv = __frcp_rn(rho);
    const int W = g.W, nout = g.nout;
    const bool att = A.last && g.ao >= 0;
    if (!g.ydir) {
        const int qn = (nout + 3) >> 2;
        for (int k = tid; k < g.count * qn; k += NTH) {
            const int s = k / qn, i = 4 * (k - s * qn);
            const float4 pv = *reinterpret_cast<const float4*>(sp + s * rc + i);
            const float* dv = reinterpret_cast<const float*>(sm + (s >> 1) * SP + W + i) + (s & 1);
            float v[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
            for (int e = 0; e < 4; e++) {
                v[e] = rk_update(v[e], dv[2 * e], g.vel, cdt, rho, c2, rinv);
                if (att && i + e < nout) v[e] = __fmul_rn(v[e], A.att[g.ao + i + e]);
            }
            float* o = out + g.fo + (long long)(job.first + s) * g.fp + i;
            if (i + 4 <= nout) {
                *reinterpret_cast<float4*>(o) = make_float4(v[0], v[1], v[2], v[3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (i + e < nout) o[e] = v[e];
            }
        }
    } else if (g.vec) {
        constexpr int G = S2 / 4;
        for (int k = tid; k < G * nout; k += NTH) {
            const int q = k % G, i = k / G;
            const float4 pv = *reinterpret_cast<const float4*>(sp + i * S2 + 4 * q);
            const float2 d0 = sm[2 * q * SP + W + i], d1 = sm[(2 * q + 1) * SP + W + i];
            float v[4] = {rk_update(pv.x, d0.x, g.vel, cdt, rho, c2, rinv), rk_update(pv.y, d0.y, g.vel, cdt, rho, c2, rinv),
                          rk_update(pv.z, d1.x, g.vel, cdt, rho, c2, rinv), rk_update(pv.w, d1.y, g.vel, cdt, rho, c2, rinv)};
            if (att) {
                const float a = A.att[g.ao + i];
#pragma unroll
                for (int e = 0; e < 4; e++) v[e] = __fmul_rn(v[e], a);
            }
            *reinterpret_cast<float4*>(out + g.fo + (long long)i * g.fp + job.first + 4 * q) =
                make_float4(v[0], v[1], v[2], v[3]);
        }
    } else {
        const float* smf = reinterpret_cast<const float*>(sm);
        for (int k = tid; k < g.count * nout; k += NTH) {
            const int s = k % g.count, i = k / g.count;
            float v = rk_update(sp[i * S2 + s], smf[2 * ((s >> 1) * SP + W + i) + (s & 1)], g.vel, cdt, rho, c2, rinv);
            if (att) v = __fmul_rn(v, A.att[g.ao + i]);
            out[g.fo + (long long)i * g.fp + job.first + s] = v;
        }
    }
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_pipe(StageArgs A, int n_jobs) {
    constexpr int NT = C::NT, S2 = 2 * C::CS;
    extern __shared__ __align__(16) float2 sm[];
    const int rc = A.row_cap;
    float* slots = reinterpret_cast<float*>(sm + C::BUF);
    const int slot_f = pipe_slot_floats(S2, rc);
    const int tid = threadIdx.x;
    const int stride = gridDim.x;
    const int mine = (int)blockIdx.x < n_jobs ? (n_jobs - 1 - (int)blockIdx.x) / stride + 1 : 0;
    // prologue: jobs 0 and 1 of this CTA in flight
    for (int k = 0; k < 2; k++) {
        if (k < mine) {
            const DevJob job = A.jobs[blockIdx.x + k * stride];
            if (!(job.kind & JK_COPY)) pipe_stage_in<C, NT>(slots + k * slot_f, A, job, rc, tid);
        }
        cp_commit();
    }
    for (int k = 0; k < mine; k++) {
        const float* slot = slots + (k & 1) * slot_f;
        cp_wait1();
        __syncthreads();
        const DevJob job = A.jobs[blockIdx.x + k * stride];
        const DevDomain dom = A.doms[job.dom];
        if (job.kind & JK_COPY) {
            copy_axis<NT>(A, dom, job.kind & JK_Y, tid);
        } else {
            const PipeJob g = pipe_job<S2>(A, job, dom, A.first_step[dom.scene] != 0);
            pipe_blend<C, NT>(sm, slot, A, job, g, rc, tid);
            __syncthreads();
            convolve<C, NT, 0, false>(sm, A.tw, A.filt + job.dtab, tid);
            __syncthreads();
            pipe_epilogue<C, NT>(sm, slot + 2 * S2 * rc, A, job, dom, g, rc, tid);
        }
        __syncthreads();   // the slot and the FFT buffer are free again
        if (k + 2 < mine) {
            const DevJob nxt = A.jobs[blockIdx.x + (k + 2) * stride];
            if (!(nxt.kind & JK_COPY)) pipe_stage_in<C, NT>(slots + (k & 1) * slot_f, A, nxt, rc, tid);
        }
        cp_commit();
    }
}

// ---------------------------------------------------------------- staged stage-start form
// The plain kernel's steps, with the stage-start values of the updated field
// (the only global reads of the epilogue) copied to shared memory by cp.async
// at the start of the job: they arrive while the strips are gathered and
// transformed, and the epilogue no longer waits on global memory.  Shared
// memory: the FFT buffer, then S2 x rc floats (rows of x jobs; [rc][S2] for y
// jobs, the layout of the pipelined form's P slot).
template <class C, int NTH>
__device__ __forceinline__ void stage_prev_in(float* sp, const StageArgs& A, const DevJob& job, const PipeJob& g,
                                              int rc, int tid) {
    constexpr int S2 = 2 * C::CS;
    const float* P = A.prev + g.fo;
    if (!g.ydir) {
        const int qp = (g.nout + 3) >> 2;   // whole quads: rows are padded past their last quad
        for (int k = tid; k < g.count * qp; k += NTH) {
            const int s = k / qp, q = k - s * qp;
            cp16(sp + s * rc + 4 * q, P + (long long)(job.first + s) * g.fp + 4 * q);
        }
    } else if (g.vec) {
        constexpr int G = S2 / 4;
        for (int k = tid; k < g.nout * G; k += NTH) {
            const int q = k % G, i = k / G;
            cp16(sp + i * S2 + 4 * q, P + (long long)i * g.fp + job.first + 4 * q);
        }
    } else {
        for (int k = tid; k < g.nout * g.count; k += NTH) {
            const int s = k % g.count, i = k / g.count;
            cp4(sp + i * S2 + s, P + (long long)i * g.fp + job.first + s);
        }
    }
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_sprev(StageArgs A) {
    extern __shared__ __align__(16) float2 sm[];
    constexpr int S2 = 2 * C::CS;
    const int rc = A.row_cap;
    float* sp = reinterpret_cast<float*>(sm + C::BUF);
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    if (job.kind & JK_COPY) {
        copy_axis<C::NT>(A, dom, job.kind & JK_Y, threadIdx.x);
        return;
    }
    const bool first = A.first_step[dom.scene] != 0;
    const PipeJob g = pipe_job<S2>(A, job, dom, first);
    stage_prev_in<C, C::NT>(sp, A, job, g, rc, threadIdx.x);
    cp_commit();
    gather<C, C::NT, false>(sm, A, job, dom, first, threadIdx.x);
    __syncthreads();
    convolve<C, C::NT, 0, false, true>(sm, A.tw, A.filt + job.dtab, threadIdx.x, 2 * job.W + g.n, job.W,
                                       job.W + g.nout);
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    pipe_epilogue<C, C::NT>(sm, sp, A, job, dom, g, rc, threadIdx.x);
}

template <class C>
size_t sprev_smem(int rc) {
    return (size_t)C::BUF * 8 + (size_t)2 * C::CS * rc * 4;
}

template <class C>
cudaError_t launch_sprev_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    static int optin = 0;
    if (optin == 0) {
        int dev;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t smem = sprev_smem<C>(a.row_cap);
    if (a.row_cap < 4 || (a.row_cap & 3) || smem > (size_t)optin) return cudaErrorInvalidValue;   // does not fit
    stage_sprev<C><<<n_jobs, C::NT, smem, st>>>(a);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_sprev_t() {
    int dev, optin;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return cudaFuncSetAttribute(stage_sprev<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <class C>
StageVariant make_sprev_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT; v.smem = 0; v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.persistent = false;
    v.pipe = true;   // needs the bucket's row cap
    v.bf16 = false;
    v.ctw = C::CTW;
    v.launch = &launch_sprev_t<C>;
    v.prepare = &prepare_sprev_t<C>;
    v.smem_for = &sprev_smem<C>;
    v.name = name;
    return v;
}

template <class C>
size_t pipe_smem(int rc) {
    return (size_t)C::BUF * 8 + 2 * (size_t)pipe_slot_floats(2 * C::CS, rc) * 4;
}

template <class C>
cudaError_t launch_pipe_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    static int sms = 0, optin = 0;
    if (sms == 0) {
        int dev;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t smem = pipe_smem<C>(a.row_cap);
    if (a.row_cap < 4 || (a.row_cap & 3) || smem > (size_t)optin) return cudaErrorInvalidValue;   // does not fit
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stage_pipe<C>, C::NT, smem);
    const int grid_max = sms * (per > 0 ? per : 1);
    const int g = n_jobs < grid_max ? n_jobs : grid_max;
    stage_pipe<C><<<g, C::NT, smem, st>>>(a, n_jobs);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_pipe_t() {
    int dev, optin;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return cudaFuncSetAttribute(stage_pipe<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <class C>
size_t plain_smem(int) {
    return (size_t)C::SMEM;
}

template <class C>
StageVariant make_pipe_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT; v.smem = 0; v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.persistent = false;
    v.pipe = true;
    v.bf16 = false;
    v.ctw = C::CTW;
    v.launch = &launch_pipe_t<C>;
    v.prepare = &prepare_pipe_t<C>;
    v.smem_for = &pipe_smem<C>;
    v.name = name;
    return v;
}

template <class C>
cudaError_t launch_stage_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    if constexpr (C::NTP > 0) {
        static int grid = 0;
        if (grid == 0) {
            int dev, sms, per;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stage_ws<C>, C::NT + C::NTP, C::SMEM);
            grid = sms * (per > 0 ? per : 1);
        }
        const int g = n_jobs < grid ? n_jobs : grid;
        stage_ws<C><<<g, C::NT + C::NTP, C::SMEM, st>>>(a, n_jobs);
    } else {
        stage_kernel<C><<<n_jobs, C::NT, C::SMEM, st>>>(a);
    }
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_stage_t() {
    if constexpr (C::NTP > 0)
        return cudaFuncSetAttribute(stage_ws<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    else
        return cudaFuncSetAttribute(stage_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
}

template <class C>
cudaError_t launch_stage_dev_t(const int* count, const StageArgs& a, int* counter, cudaStream_t st) {
    static int grid = 0;
    if (grid == 0) {
        int dev, sms, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stage_kernel_dev<C>, C::NT, C::SMEM);
        grid = sms * (per > 0 ? per : 1);
    }
    stage_kernel_dev<C><<<grid, C::NT, C::SMEM, st>>>(a, count, counter);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_stage_dev_t() {
    return cudaFuncSetAttribute(stage_kernel_dev<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
}

template <class C>
StageVariant make_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT + C::NTP; v.smem = C::SMEM; v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.persistent = C::NTP > 0;
    v.pipe = false;
    v.bf16 = C::TC != 0;
    v.ctw = C::CTW;
    v.launch = &launch_stage_t<C>;
    v.prepare = &prepare_stage_t<C>;
    v.smem_for = &plain_smem<C>;
    v.name = name;
    return v;
}

// a plain variant that also has the device-count persistent form
template <class C>
StageVariant make_dev_variant(const char* name) {
    static_assert(C::NTP == 0 && C::TC == 0, "the device-count form runs the plain stage kernel");
    StageVariant v = make_variant<C>(name);
    v.launch_dev = &launch_stage_dev_t<C>;
    v.prepare_dev = &prepare_stage_dev_t<C>;
    return v;
}

}  // namespace pstd
