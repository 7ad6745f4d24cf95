// stage_tc5.cuh -- precision study: the radix-16 DFT passes of long strips as
// tcgen05 (5th-generation tensor core) GEMMs with TMEM accumulators.
//
// Same decomposition as the mma.sync study of stage_kernel.cuh (*_pass_tc):
// 128 butterflies of a radix-16 pass form the rows of a real GEMM
//   [Re x | Im x] (128 x 32) * F (32 x 32) = [Re X | Im X],
// F = [[C, -S], [S, C]] (C = cos 2 pi q k / 16, S = sin ...) for the forward
// transform, [[C, S], [-S, C]] for the inverse.  Operands are TF32 (kind::tf32,
// FP32 accumulation) split three ways: x = x_hi + x_lo with x_hi = tf32(x),
// x_lo = tf32(x - x_hi), and the product summed as x_hi F_hi + x_hi F_lo +
// x_lo F_hi (about 2^-21 relative, the x_lo F_lo term dropped).
//
// Per group of 128 butterflies: all threads gather the butterflies from the
// shared-memory strip, split them and store A_hi / A_lo in the canonical
// K-major layout without swizzle (8-row x 16-byte core matrices; core
// matrices along K 128 bytes apart, 8-row groups 1024 bytes apart); one
// thread issues the 12 tcgen05.mma (K = 8 each) into two 128-lane x
// 32-column TMEM accumulators (the hi x hi term, and the two cross terms
// apart) and commits them to an mbarrier; warps 0-3 read their 32 lanes back
// with tcgen05.ld (one butterfly's 32 outputs per thread), add the two
// accumulators in FP32, apply the pass twiddles and scatter to the strip.  Every mbarrier wait is bounded;
// on a timeout the CTA records error 2 in *A.err, frees its TMEM and leaves.
#pragma once
#include "stage_tma.cuh"

namespace pstd {

// ---------------------------------------------------------------- PTX
__device__ __forceinline__ uint32_t f32_to_tf32(float x) {   // round to nearest (ties away), TF32 in a b32
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// shared-memory matrix descriptor: K-major, no swizzle, version 1
__device__ __forceinline__ uint64_t umma_desc(const void* tile, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = (uint64_t)((smem_addr(tile) >> 4) & 0x3FFF);
    return a | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::tf32: D F32, A and B TF32 K-major, N, M
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
    return (1u << 4)                      // D format F32
           | (2u << 7) | (2u << 10)       // A, B format TF32
           | ((uint32_t)(N >> 3) << 17)   // N / 8
           | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive TMEM columns of this thread's lane (warp w reads lanes 32 (w % 4) ..)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- operand tiles
// Operand tile of R rows x 32 TF32 (K): element (row, k) at
//   (row / 8) * 1024 + (k / 4) * 128 + (row % 8) * 16 + (k % 4) * 4 bytes
__device__ __forceinline__ int tile_off(int row, int k) {
    return (row >> 3) * 256 + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);   // in 4-byte words
}
constexpr uint32_t TC5_LBO = 128, TC5_SBO = 1024;
constexpr int TC5_ROWS = 128;                     // butterflies per GEMM group (M)
constexpr int TC5_A_WORDS = TC5_ROWS * 32;        // one A tile (16 KB)
constexpr int TC5_B_WORDS = 32 * 32;              // one B tile (4 KB)

// The four B tiles (forward hi / lo, inverse hi / lo), N x K (K-major):
// B[n][k] = F[k][n] of the forward / inverse real DFT-16 matrix.
__device__ __forceinline__ float dft16_real(int k, int n, bool inv) {
    // F[k][n]: k, n < 16 -> Re parts; >= 16 -> Im parts
    const int q = k & 15, m = n & 15;
    const float c = cos16((q * m) & 15), s = sin16((q * m) & 15);
    const bool ki = k >= 16, ni = n >= 16;
    if (ki == ni) return c;
    // forward: Re out gets +S b (k Im, n Re), Im out gets -S a (k Re, n Im)
    const float v = ki ? s : -s;
    return inv ? -v : v;
}

__device__ inline void tc5_build_b(uint32_t* b, int tid, int nth) {
    for (int i = tid; i < 4 * TC5_B_WORDS; i += nth) {
        const int t = i / TC5_B_WORDS, e = i - t * TC5_B_WORDS;
        const int n = e / 32, k = e % 32;
        const float f = dft16_real(k, n, t >= 2);
        const uint32_t hi = f32_to_tf32(f);
        const uint32_t w = (t & 1) ? f32_to_tf32(f - __uint_as_float(hi)) : hi;
        b[t * TC5_B_WORDS + tile_off(n, k)] = w;
    }
}

struct Tc5 {
    uint32_t* a_hi;
    uint32_t* a_lo;
    const uint32_t* b;   // 4 tiles
    uint64_t* bar;
    uint32_t tmem;
    uint32_t phase;
    int* err;
    bool ok;
};

// one GEMM group: A (already stored) x F -> TMEM, all threads wait for it
template <int NTH>
__device__ __forceinline__ bool tc5_gemm(Tc5& t, bool inv, int tid) {
    fence_async_smem();   // the A tiles written by this CTA's threads, seen by the tensor core
    __syncthreads();
    if (tid == 0) {
        tc_fence_after();
        constexpr uint32_t idesc = umma_idesc_tf32(TC5_ROWS, 32);
        const uint32_t* bh = t.b + (inv ? 2 : 0) * TC5_B_WORDS;
        const uint32_t* bl = bh + TC5_B_WORDS;
        uint32_t acc = 0;
        // the cross terms (about 2^-11 of the hi x hi term) accumulate apart,
        // in columns 32..63, so that the tensor core's accumulation of the
        // large term does not round them away; the two are added in FP32
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {   // K = 8 per instruction: two core matrices
            const uint64_t ah = umma_desc(t.a_hi + ks * 64, TC5_LBO, TC5_SBO);
            const uint64_t al = umma_desc(t.a_lo + ks * 64, TC5_LBO, TC5_SBO);
            const uint64_t dh = umma_desc(bh + ks * 64, TC5_LBO, TC5_SBO);
            const uint64_t dl = umma_desc(bl + ks * 64, TC5_LBO, TC5_SBO);
            umma_tf32(t.tmem + 32, al, dh, idesc, acc);
            umma_tf32(t.tmem + 32, ah, dl, idesc, 1);
            umma_tf32(t.tmem, ah, dh, idesc, acc);
            acc = 1;
        }
        umma_commit(t.bar);
    }
    const bool ok = __syncthreads_and(mbar_wait(t.bar, t.phase)) != 0;
    if (ok) t.phase ^= 1;   // on a timeout the phase stays pending (waited for again before TMEM is freed)
    tc_fence_after();
    return ok;
}

// store butterfly `row` (16 complex values x) of the group as A rows, split
__device__ __forceinline__ void tc5_store_row(Tc5& t, int row, const float2 (&x)[16]) {
#pragma unroll
    for (int q = 0; q < 16; q++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float v = h ? x[q].y : x[q].x;
            const uint32_t hi = f32_to_tf32(v);
            const int o = tile_off(row, q + 16 * h);
            t.a_hi[o] = hi;
            t.a_lo[o] = f32_to_tf32(v - __uint_as_float(hi));
        }
    }
}

// read back butterfly `row` (warps 0-3 only, row = tid): X[k] = (col k, col 16 + k)
__device__ __forceinline__ void tc5_load_row(const Tc5& t, int warp, float2 (&y)[16]) {
    float big[32], small[32];
    const uint32_t lane = (uint32_t)(32 * (warp & 3)) << 16;
    tmem_ld32(t.tmem + lane, big);
    tmem_ld32(t.tmem + lane + 32, small);
#pragma unroll
    for (int k = 0; k < 16; k++) y[k] = make_float2(small[k] + big[k], small[16 + k] + big[16 + k]);
}

// forward (DIF) radix-16 pass of block size M on tensor cores: DFT then twiddle
template <class C, int M, int TOFF, int NTH>
__device__ __forceinline__ bool fwd_pass_tc5(float2* sm, const float2* tw, Tc5& t, int tid) {
    constexpr int Q = M / 16, ITEMS = C::CS * (C::L / 16);
    static_assert(ITEMS % TC5_ROWS == 0 && NTH >= TC5_ROWS, "whole GEMM groups");
    for (int g0 = 0; g0 < ITEMS; g0 += TC5_ROWS) {
        for (int r = tid; r < TC5_ROWS; r += NTH) {
            int n1;
            float2* base = pass_base<C, 16, M>(sm, g0 + r, n1);
            float2 x[16];
#pragma unroll
            for (int q = 0; q < 16; q++) x[q] = base[q * Q];
            tc5_store_row(t, r, x);
        }
        if (!tc5_gemm<NTH>(t, false, tid)) return false;
        if (tid < TC5_ROWS) {
            int n1;
            float2* base = pass_base<C, 16, M>(sm, g0 + tid, n1);
            float2 y[16];
            tc5_load_row(t, tid >> 5, y);
            if (Q > 1) {
                float2 w[16];
                load_twiddles<16, false>(tw + TOFF + n1 * 16, w);
#pragma unroll
                for (int k = 1; k < 16; k++) y[k] = cmul(y[k], w[k]);
            }
#pragma unroll
            for (int k = 0; k < 16; k++) base[k * Q] = y[k];
        }
        tc_fence_before();
        __syncthreads();   // TMEM read and strip writes done before the next group
    }
    return true;
}

// inverse (DIT) radix-16 pass: conjugate twiddles then inverse DFT
template <class C, int M, int TOFF, int NTH>
__device__ __forceinline__ bool inv_pass_tc5(float2* sm, const float2* tw, Tc5& t, int tid) {
    constexpr int Q = M / 16, ITEMS = C::CS * (C::L / 16);
    static_assert(ITEMS % TC5_ROWS == 0 && NTH >= TC5_ROWS, "whole GEMM groups");
    for (int g0 = 0; g0 < ITEMS; g0 += TC5_ROWS) {
        for (int r = tid; r < TC5_ROWS; r += NTH) {
            int n1;
            float2* base = pass_base<C, 16, M>(sm, g0 + r, n1);
            float2 x[16];
#pragma unroll
            for (int q = 0; q < 16; q++) x[q] = base[q * Q];
            if (Q > 1) {
                float2 w[16];
                load_twiddles<16, false>(tw + TOFF + n1 * 16, w);
#pragma unroll
                for (int k = 1; k < 16; k++) x[k] = cmulc(x[k], w[k]);
            }
            tc5_store_row(t, r, x);
        }
        if (!tc5_gemm<NTH>(t, true, tid)) return false;
        if (tid < TC5_ROWS) {
            int n1;
            float2* base = pass_base<C, 16, M>(sm, g0 + tid, n1);
            float2 y[16];
            tc5_load_row(t, tid >> 5, y);
#pragma unroll
            for (int k = 0; k < 16; k++) base[k * Q] = y[k];
        }
        tc_fence_before();
        __syncthreads();
    }
    return true;
}

// radix plan 16.16.16.R3 (R3 on CUDA cores, in the mid pass)
template <class C, int NTH>
__device__ __forceinline__ bool convolve_tc5(float2* sm, const float2* tw, const float2* filt, Tc5& t, int tid) {
    static_assert(C::R0 == 16 && C::R1 == 16 && C::R2 == 16 && C::NP == 4, "radix plan 16.16.16.R3");
    constexpr int M0 = C::L, M1 = C::M1, M2 = C::M2, T1 = C::T1, T2 = C::T2;
    if (!fwd_pass_tc5<C, M0, 0, NTH>(sm, tw, t, tid)) return false;
    if (!fwd_pass_tc5<C, M1, T1, NTH>(sm, tw, t, tid)) return false;
    if (!fwd_pass_tc5<C, M2, T2, NTH>(sm, tw, t, tid)) return false;
    mid_pass<C, C::R3, NTH, false>(sm, filt, tid);
    __syncthreads();
    if (!inv_pass_tc5<C, M2, T2, NTH>(sm, tw, t, tid)) return false;
    if (!inv_pass_tc5<C, M1, T1, NTH>(sm, tw, t, tid)) return false;
    return inv_pass_tc5<C, M0, 0, NTH>(sm, tw, t, tid);
}

template <class C>
__global__ void __launch_bounds__(C::NT, 1) stage_tc5(StageArgs A) {
    extern __shared__ __align__(16) float2 sm[];
    constexpr int NT = C::NT;
    // strips, then (128-byte aligned) A_hi, A_lo, the four B tiles, mbarrier, TMEM address
    unsigned char* base = reinterpret_cast<unsigned char*>(sm) + (size_t)C::BUF * 8;
    base += (128u - (smem_addr(base) & 127u)) & 127u;
    Tc5 t;
    t.a_hi = reinterpret_cast<uint32_t*>(base);
    t.a_lo = t.a_hi + TC5_A_WORDS;
    uint32_t* b = t.a_lo + TC5_A_WORDS;
    t.b = b;
    t.bar = reinterpret_cast<uint64_t*>(b + 4 * TC5_B_WORDS);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(t.bar + 1);
    t.phase = 0;
    t.err = A.err;
    const int tid = threadIdx.x, warp = tid >> 5;
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    if (job.kind & JK_COPY) {
        copy_axis<NT>(A, dom, job.kind & JK_Y, tid);
        return;
    }
    tc5_build_b(b, tid, NT);
    if (tid == 0) {
        mbar_init(t.bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_addr(tslot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    t.tmem = *tslot;
    const bool first = A.first_step[dom.scene] != 0;
    gather<C, NT, true>(sm, A, job, dom, first, tid);
    __syncthreads();
    const bool ok = convolve_tc5<C, NT>(sm, A.tw, A.filt + job.dtab, t, tid);
    if (ok) {
        __syncthreads();
        epilogue<C, NT>(sm, A, job, dom, tid);
    } else if (tid == 0) {
        if (A.err) atomicExch(A.err, 2);
        mbar_wait(t.bar, t.phase);   // bounded: the group's MMAs, before their TMEM is freed
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(t.tmem) : "memory");
}

template <class C>
constexpr size_t tc5_smem() {
    return (size_t)C::BUF * 8 + 128 + (size_t)(2 * TC5_A_WORDS + 4 * TC5_B_WORDS) * 4 + 16;
}

template <class C>
cudaError_t launch_tc5_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    stage_tc5<C><<<n_jobs, C::NT, tc5_smem<C>(), st>>>(a);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_tc5_t() {
    return cudaFuncSetAttribute(stage_tc5<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc5_smem<C>());
}

template <class C>
size_t tc5_smem_for(int) {
    return tc5_smem<C>();
}

template <class C>
StageVariant make_tc5_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT; v.smem = (int)tc5_smem<C>(); v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.persistent = false;
    v.pipe = false;
    v.bf16 = true;   // a precision-study form: never tuned, chosen by PSTD_DFT
    v.tc5 = true;
    v.launch = &launch_tc5_t<C>;
    v.prepare = &prepare_tc5_t<C>;
    v.smem_for = &tc5_smem_for<C>;
    v.name = name;
    return v;
}

}  // namespace pstd
