// stage_tma.cuh -- the TMA-staged persistent form of the stage kernel.
//
// Same arithmetic as stage_kernel (kernel/core/kernel_functions.cpp:123-318
// fused with kernel/Solver.cpp:162-182), but no warp waits on global memory
// for a job's strips or stage-start values: one thread of each persistent CTA
// hands the copy engine (TMA) the NEXT job's inputs while the warps transform
// the current one.
//
//   raw region  A, B : the strips of the derivative input (A = px / vx / vy /
//                      stale p0, B = py when p0 is formed as px + py);
//   prev region P    : the stage-start values of the field the job updates;
//   bands            : the blended interface bands (plain loads: 2W values
//                      per strip).
//
// Row (x) jobs stage each row with one bulk copy (cp.async.bulk, rows are
// 128-byte aligned and padded to whole 16-byte quads).  Column (y) jobs stage
// [rows x 4 columns] boxes through a 2-D tensor map per (domain, field, state
// set) (cp.async.bulk.tensor.2d): the region holds [column group][row][4].
// Each region completes on its own mbarrier (expect_tx bytes); the raw region
// of job k+1 is issued as soon as job k has been blended into the transform
// buffer, the prev region as soon as job k's epilogue has read it.
//
// Every mbarrier wait is bounded (about a second of clock cycles): on a
// timeout the CTA records PSTD stage error 1 in *A.err, waits (again bounded)
// for its copies in flight and returns; the host reports the error.
//
// Column jobs whose first column is not a multiple of four (the first job of
// a ragged run) cannot start a tensor box on a 16-byte boundary: they take
// the plain gather / epilogue of stage_kernel.
#pragma once
#include "stage_fused.cuh"

namespace pstd {

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false after about 2^31 clock cycles (~1 s at 2 GHz)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > (1LL << 31)) return false;
    return true;
}
// generic-proxy accesses of shared memory before async-proxy (TMA) writes
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// bytes (multiple of 16) from global to shared, both 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// one box of a 2-D tensor map at element coordinates (x = column, y = row);
// x * 4 bytes must be a multiple of 16 (callers start boxes at columns 4k)
__device__ __forceinline__ void tma_box_2d(void* dst, const void* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// ---------------------------------------------------------------- geometry
// floats staged per strip: whole 16-byte quads of a row job's strips, and
// whole boxes of a column job's strips (box rows min(256, rows rounded to 8))
// a region holds S2 rows of a row job or ceil(S2 / 4) column groups of 4
__host__ __device__ constexpr size_t tma_region_bytes(int S2, int rc) {
    return ((size_t)((S2 + 3) / 4 * 4) * tma_cap(rc) * 4 + 127) / 128 * 128;
}

// tensor map index: field 0 px, 1 py, 2 vx, 3 vy in state set 0..2; the
// stale / initial p0 array as field 0 of "set" 3
__device__ __forceinline__ const void* tma_map(const StageArgs& A, int dom, int field, int set) {
    return A.maps + (size_t)((dom * 4 + field) * 4 + set) * PSTD_TMAP_BYTES;
}

// what one job stages
struct TmaJob {
    bool vel, ydir, stale, two;
    int n;       // strip length of the derivative input
    int nout;    // outputs per strip
    int rows_in, rows_prev;   // column jobs: rows of the input / updated field
};

__device__ __forceinline__ TmaJob tma_job(const StageArgs& A, const DevJob& job, const DevDomain& dom, bool first) {
    TmaJob t;
    t.vel = job.kind & JK_VEL;
    t.ydir = job.kind & JK_Y;
    t.stale = !t.vel && A.stage == 0 && (dom.pml || first);
    t.two = !t.vel && !t.stale;
    t.n = (t.ydir ? dom.ny : dom.nx) + (t.vel ? 1 : 0);
    t.nout = t.vel ? t.n - 1 : t.n + 1;
    t.rows_in = t.n;        // column jobs: the strip runs along the rows
    t.rows_prev = t.nout;
    return t;
}

// a column job can start its boxes on 16-byte boundaries
__device__ __forceinline__ bool tma_eligible(const DevJob& job) {
    return !(job.kind & JK_COPY) && (!(job.kind & JK_Y) || (job.first & 3) == 0);
}

// issue the raw (input) copies of one job into regions ra, rb (thread 0)
template <int S2>
__device__ __forceinline__ void tma_issue_raw(float* ra, float* rb, uint64_t* bar, const StageArgs& A,
                                              const DevJob& job, int cap) {
    const DevDomain dom = A.doms[job.dom];
    const TmaJob t = tma_job(A, job, dom, A.first_step[dom.scene] != 0);
    const int nf = t.two ? 2 : 1;
    if (!t.ydir) {
        const uint32_t bytes = (uint32_t)((t.n + 3) / 4 * 16);
        mbar_expect_tx(bar, bytes * nf * job.count);
        const float* fa;
        int pitch;
        if (t.vel) { fa = A.in + dom.o_vx; pitch = dom.pitch_vx; }
        else if (t.stale) { fa = A.p0 + dom.o_p0; pitch = dom.pitch_p; }
        else { fa = A.in + dom.o_px; pitch = dom.pitch_p; }
        const float* fb = A.in + dom.o_py;
        for (int s = 0; s < job.count; s++) {
            const long long r = (long long)(job.first + s) * pitch;
            bulk_g2s(ra + s * cap, fa + r, bytes, bar);
            if (nf == 2) bulk_g2s(rb + s * cap, fb + r, bytes, bar);
        }
    } else {
        const int BR = tma_box_rows(t.rows_in), nbox = (t.rows_in + BR - 1) / BR;
        const int G = (job.count + 3) / 4;
        mbar_expect_tx(bar, (uint32_t)(nf * G * nbox * BR * 16));
        const void* ma = t.vel ? tma_map(A, job.dom, 3, A.set_in) : t.stale ? tma_map(A, job.dom, 0, 3)
                                                                               : tma_map(A, job.dom, 0, A.set_in);
        const void* mb = tma_map(A, job.dom, 1, A.set_in);
        for (int g = 0; g < G; g++)
            for (int b = 0; b < nbox; b++) {
                tma_box_2d(ra + (g * cap + b * BR) * 4, ma, job.first + 4 * g, b * BR, bar);
                if (nf == 2) tma_box_2d(rb + (g * cap + b * BR) * 4, mb, job.first + 4 * g, b * BR, bar);
            }
    }
}

// issue the stage-start copies of the field one job updates (thread 0)
template <int S2>
__device__ __forceinline__ void tma_issue_prev(float* rp, uint64_t* bar, const StageArgs& A, const DevJob& job,
                                               int cap) {
    const DevDomain dom = A.doms[job.dom];
    const bool vel = job.kind & JK_VEL, ydir = job.kind & JK_Y;
    if (!ydir) {
        // vel: px (nx per row); else vx (nx + 1 per row)
        const int len = vel ? dom.nx : dom.nx + 1;
        const uint32_t bytes = (uint32_t)((len + 3) / 4 * 16);
        mbar_expect_tx(bar, bytes * job.count);
        const float* f = A.prev + (vel ? dom.o_px : dom.o_vx);
        const int pitch = vel ? dom.pitch_p : dom.pitch_vx;
        for (int s = 0; s < job.count; s++) bulk_g2s(rp + s * cap, f + (long long)(job.first + s) * pitch, bytes, bar);
    } else {
        // vel: py (ny rows); else vy (ny + 1 rows)
        const int rows = vel ? dom.ny : dom.ny + 1;
        const int BR = tma_box_rows(rows), nbox = (rows + BR - 1) / BR;
        const int G = (job.count + 3) / 4;
        mbar_expect_tx(bar, (uint32_t)(G * nbox * BR * 16));
        const void* m = tma_map(A, job.dom, vel ? 1 : 3, A.set_prev);
        for (int g = 0; g < G; g++)
            for (int b = 0; b < nbox; b++) tma_box_2d(rp + (g * cap + b * BR) * 4, m, job.first + 4 * g, b * BR, bar);
    }
}

// ---------------------------------------------------------------- blend
// staged strips (+ p0 = px + py) and bands -> the complex strips of the
// transform buffer, positions [0, 2W + n) (the pruned first pass reads no
// further); strips past the job's count are zero, as in stage_kernel
template <class C, int NTH>
__device__ __forceinline__ void tma_blend(float2* sm, const float* ra, const float* rb, const float* sband,
                                          const DevJob& job, const TmaJob& t, int cap, int tid) {
    constexpr int CS = C::CS, SP = C::SP, S2 = 2 * CS, BAND = 64;
    const int W = job.W, n = t.n, count = job.count;
    if (!t.ydir) {
        const int chunks = (n + 3) >> 2;
        const bool pair16 = (SP % 2 == 0) && !(W & 1);   // 16-byte aligned pairs in shared memory
        for (int it = tid; it < CS * chunks; it += NTH) {
            const int cs = it / chunks, i = (it - cs * chunks) << 2;
            const int s0 = 2 * cs;
            float4 u = make_float4(0.f, 0.f, 0.f, 0.f), v = u;
            if (s0 < count) {
                u = *reinterpret_cast<const float4*>(ra + s0 * cap + i);
                if (t.two) u = add4(u, *reinterpret_cast<const float4*>(rb + s0 * cap + i));
            }
            if (s0 + 1 < count) {
                v = *reinterpret_cast<const float4*>(ra + (s0 + 1) * cap + i);
                if (t.two) v = add4(v, *reinterpret_cast<const float4*>(rb + (s0 + 1) * cap + i));
            }
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
    } else {
        constexpr int GT = (S2 + 3) / 4;   // column groups of the job
        for (int i = tid; i < n; i += NTH) {
#pragma unroll
            for (int g = 0; g < GT; g++) {
                float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
                if (4 * g < count) {
                    u = *reinterpret_cast<const float4*>(ra + (g * cap + i) * 4);
                    if (t.two) u = add4(u, *reinterpret_cast<const float4*>(rb + (g * cap + i) * 4));
                    if (4 * g + 1 >= count) u.y = 0.f;
                    if (4 * g + 2 >= count) u.z = 0.f;
                    if (4 * g + 3 >= count) u.w = 0.f;
                }
                sm[(2 * g) * SP + W + i] = make_float2(u.x, u.y);
                if (2 * g + 1 < CS) sm[(2 * g + 1) * SP + W + i] = make_float2(u.z, u.w);
            }
        }
    }
    // interface bands: positions [0, W) and [W + n, 2W + n)
    for (int idx = tid; idx < CS * 2 * W; idx += NTH) {
        const int cs = idx / (2 * W), j = idx - cs * (2 * W);
        const int p = j < W ? j : n + j;
        sm[cs * SP + p] = make_float2(sband[2 * cs * BAND + j], sband[(2 * cs + 1) * BAND + j]);
    }
}

// ---------------------------------------------------------------- epilogue
// slice [W, W + nout), RK update against the staged stage-start values,
// (sixth stage) PML multiply of vx / vy, store
template <class C, int NTH, bool VEL, bool ATT>
__device__ __forceinline__ void tma_epilogue_k(const float2* sm, const float* rp, const StageArgs& A,
                                               const DevJob& job, const DevDomain& dom, const TmaJob& t, int cap,
                                               int tid) {
    constexpr int CS = C::CS, SP = C::SP, S2 = 2 * CS;
    float* __restrict__ out = A.out;
    const int W = job.W, nout = t.nout, count = job.count;
    const float cdt = A.doms[job.dom].cdt[A.stage];
    const float rho = dom.rho, c2 = dom.c2, rinv = __frcp_rn(rho);
    long long fo;
    int fp, ao;
    if (!VEL) {
        fo = t.ydir ? dom.o_vy : dom.o_vx;
        fp = t.ydir ? dom.pitch_vy : dom.pitch_vx;
        ao = t.ydir ? dom.att_yv : dom.att_xv;
    } else {
        fo = t.ydir ? dom.o_py : dom.o_px;
        fp = dom.pitch_p;
        ao = -1;
    }
    if (!t.ydir) {
        const int chunks = (nout + 3) >> 2;
        const bool pair16 = (SP % 2 == 0) && !(W & 1);
        for (int it = tid; it < CS * chunks; it += NTH) {
            const int cs = it / chunks, i = (it - cs * chunks) << 2;
            const int s0 = 2 * cs;
            if (s0 >= count) continue;
            const bool h1 = s0 + 1 < count;
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
                const float4 pv = *reinterpret_cast<const float4*>(rp + (s0 + h) * cap + i);
                float v[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    v[e] = rk_update(v[e], h ? d[e].y : d[e].x, VEL, cdt, rho, c2, rinv);
                    if (ATT && i + e < nout) v[e] = __fmul_rn(v[e], __ldg(A.att + ao + i + e));
                }
                float* o = out + fo + (long long)(job.first + s0 + h) * fp + i;
                if (i + 4 <= nout) {
                    *reinterpret_cast<float4*>(o) = make_float4(v[0], v[1], v[2], v[3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; e++)
                        if (i + e < nout) o[e] = v[e];
                }
            }
        }
    } else {
        constexpr int GT = (S2 + 3) / 4;
        for (int i = tid; i < nout; i += NTH) {
            const float a = ATT ? __ldg(A.att + ao + i) : 1.f;
#pragma unroll
            for (int g = 0; g < GT; g++) {
                if (4 * g >= count) break;
                const float4 pv = *reinterpret_cast<const float4*>(rp + (g * cap + i) * 4);
                const float2 d0 = sm[(2 * g) * SP + W + i];
                const float2 d1 = (2 * g + 1 < CS) ? sm[(2 * g + 1) * SP + W + i] : make_float2(0.f, 0.f);
                float v[4] = {rk_update(pv.x, d0.x, VEL, cdt, rho, c2, rinv), rk_update(pv.y, d0.y, VEL, cdt, rho, c2, rinv),
                              rk_update(pv.z, d1.x, VEL, cdt, rho, c2, rinv), rk_update(pv.w, d1.y, VEL, cdt, rho, c2, rinv)};
                if (ATT) {
#pragma unroll
                    for (int e = 0; e < 4; e++) v[e] = __fmul_rn(v[e], a);
                }
                float* o = out + fo + (long long)i * fp + job.first + 4 * g;
                if (4 * g + 4 <= count) {
                    *reinterpret_cast<float4*>(o) = make_float4(v[0], v[1], v[2], v[3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; e++)
                        if (4 * g + e < count) o[e] = v[e];
                }
            }
        }
    }
}

template <class C, int NTH>
__device__ __forceinline__ void tma_epilogue(const float2* sm, const float* rp, const StageArgs& A, const DevJob& job,
                                             const DevDomain& dom, const TmaJob& t, int cap, int tid) {
    const int ao = t.ydir ? dom.att_yv : dom.att_xv;
    if (t.vel) tma_epilogue_k<C, NTH, true, false>(sm, rp, A, job, dom, t, cap, tid);
    else if (A.last && ao >= 0) tma_epilogue_k<C, NTH, false, true>(sm, rp, A, job, dom, t, cap, tid);
    else tma_epilogue_k<C, NTH, false, false>(sm, rp, A, job, dom, t, cap, tid);
}

// blended band values of every real strip ([strip][2W], low band then high
// band) -- plain loads, issued before the staged strips are waited for
template <class C, int NTH>
__device__ __forceinline__ void tma_bands(float (&bv)[(2 * C::CS * 64 + NTH - 1) / NTH], const StageArgs& A,
                                          const DevJob& job, const DevDomain& dom, const TmaJob& t, bool first, int tid) {
    constexpr int S2 = 2 * C::CS, BPT = (S2 * 64 + NTH - 1) / NTH;
    const int W = job.W;
    const Src S = strip_source(A, dom, t.vel, t.ydir, first);
    const FusedBands B = fused_bands(A, job, t.vel, t.ydir, first);
#pragma unroll
    for (int k = 0; k < BPT; k++) {
        const int idx = threadIdx.x + k * NTH;
        const int s = idx / (2 * W), j = idx - s * (2 * W);
        float v = 0.f;
        if (idx < S2 * 2 * W && s < job.count) {
            const int p = j < W ? j : t.n + j;
            if (t.ydir) v = t.vel ? fused_band<true, true>(job, S, B, t.n, s, p) : fused_band<true, false>(job, S, B, t.n, s, p);
            else v = t.vel ? fused_band<false, true>(job, S, B, t.n, s, p) : fused_band<false, false>(job, S, B, t.n, s, p);
        }
        bv[k] = v;
    }
    (void)tid;
}

// ---------------------------------------------------------------- kernel
// transform buffer, then (from the next 128-byte boundary: tensor copies land
// on 128-byte aligned shared addresses) the three regions, bands, mbarriers
template <class C>
__host__ __device__ constexpr size_t tma_smem_bytes(int rc) {
    return (size_t)C::BUF * 8 + 128 + 3 * tma_region_bytes(2 * C::CS, rc) + (size_t)2 * C::CS * 64 * 4 + 16;
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_tma(StageArgs A, int n_jobs) {
    constexpr int NT = C::NT, S2 = 2 * C::CS, BPT = (S2 * 64 + NT - 1) / NT;
    extern __shared__ __align__(16) float2 sm[];
    const int cap = tma_cap(A.row_cap);
    const size_t rbytes = tma_region_bytes(S2, A.row_cap);
    unsigned char* base = reinterpret_cast<unsigned char*>(sm) + (size_t)C::BUF * 8;
    base += (128u - (smem_addr(base) & 127u)) & 127u;
    float* ra = reinterpret_cast<float*>(base);
    float* rb = reinterpret_cast<float*>(base + rbytes);
    float* rp = reinterpret_cast<float*>(base + 2 * rbytes);
    float* sband = reinterpret_cast<float*>(base + 3 * rbytes);
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + 3 * rbytes + (size_t)S2 * 64 * 4);
    const int tid = threadIdx.x, stride = gridDim.x;
    const int mine = (int)blockIdx.x < n_jobs ? (n_jobs - 1 - (int)blockIdx.x) / stride + 1 : 0;
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t ph_raw = 0, ph_prev = 0;
    bool raw_pending = false, prev_pending = false;   // uniform over the CTA
    if (mine > 0 && tma_eligible(A.jobs[blockIdx.x])) {
        if (tid == 0) {
            const DevJob j0 = A.jobs[blockIdx.x];
            tma_issue_raw<S2>(ra, rb, &bars[0], A, j0, cap);
            tma_issue_prev<S2>(rp, &bars[1], A, j0, cap);
        }
        raw_pending = prev_pending = true;
    }
    for (int k = 0; k < mine; k++) {
        const DevJob job = A.jobs[blockIdx.x + k * stride];
        const DevDomain dom = A.doms[job.dom];
        const bool next_tma = k + 1 < mine && tma_eligible(A.jobs[blockIdx.x + (k + 1) * stride]);
        if (!tma_eligible(job)) {
            if (job.kind & JK_COPY) {
                copy_axis<NT>(A, dom, job.kind & JK_Y, tid);
            } else {
                const bool first = A.first_step[dom.scene] != 0;
                gather<C, NT, false>(sm, A, job, dom, first, tid);
                __syncthreads();
                const bool vel = job.kind & JK_VEL;
                const int n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
                convolve<C, NT, 0, false, true>(sm, A.tw, A.filt + job.dtab, tid, 2 * job.W + n, job.W,
                                                job.W + (vel ? n - 1 : n + 1));
                __syncthreads();
                epilogue<C, NT>(sm, A, job, dom, tid);
            }
            __syncthreads();
            if (next_tma) {
                if (tid == 0) {
                    const DevJob nx = A.jobs[blockIdx.x + (k + 1) * stride];
                    fence_async_smem();
                    tma_issue_raw<S2>(ra, rb, &bars[0], A, nx, cap);
                    tma_issue_prev<S2>(rp, &bars[1], A, nx, cap);
                }
                raw_pending = prev_pending = true;
            }
            continue;
        }
        const bool first = A.first_step[dom.scene] != 0;
        const TmaJob t = tma_job(A, job, dom, first);
        float bv[BPT];
        tma_bands<C, NT>(bv, A, job, dom, t, first, tid);
        bool ok = mbar_wait(&bars[0], ph_raw);
#pragma unroll
        for (int q = 0; q < BPT; q++) {
            const int idx = tid + q * NT;
            if (idx < S2 * 2 * job.W) sband[(idx / (2 * job.W)) * 64 + idx % (2 * job.W)] = bv[q];
        }
        if (__syncthreads_or(!ok)) goto fail;
        ph_raw ^= 1;
        raw_pending = false;
        tma_blend<C, NT>(sm, ra, rb, sband, job, t, cap, tid);
        __syncthreads();
        if (next_tma) {
            if (tid == 0) {
                fence_async_smem();
                tma_issue_raw<S2>(ra, rb, &bars[0], A, A.jobs[blockIdx.x + (k + 1) * stride], cap);
            }
            raw_pending = true;
        }
        convolve<C, NT, 0, false, true>(sm, A.tw, A.filt + job.dtab, tid, 2 * job.W + t.n, job.W, job.W + t.nout);
        ok = mbar_wait(&bars[1], ph_prev);
        if (__syncthreads_or(!ok)) goto fail;
        ph_prev ^= 1;
        prev_pending = false;
        tma_epilogue<C, NT>(sm, rp, A, job, dom, t, cap, tid);
        __syncthreads();
        if (next_tma) {
            if (tid == 0) {
                fence_async_smem();
                tma_issue_prev<S2>(rp, &bars[1], A, A.jobs[blockIdx.x + (k + 1) * stride], cap);
            }
            prev_pending = true;
        }
    }
    return;
fail:
    // a staged copy did not complete in time: record it, give the copies in
    // flight a bounded wait of their own, and leave
    if (tid == 0) {
        atomicExch(A.err, 1);
        if (raw_pending) mbar_wait(&bars[0], ph_raw);
        if (prev_pending) mbar_wait(&bars[1], ph_prev);
    }
}

template <class C>
size_t tma_smem(int rc) {
    return tma_smem_bytes<C>(rc);
}

template <class C>
cudaError_t launch_tma_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    static int sms = 0, optin = 0;
    if (sms == 0) {
        int dev;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t smem = tma_smem_bytes<C>(a.row_cap);
    // the staged form needs the tensor maps, an error word and a row cap that fits
    if (!a.maps || !a.err || a.row_cap < 4 || (a.row_cap & 3) || smem > (size_t)optin) return cudaErrorInvalidValue;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stage_tma<C>, C::NT, smem);
    const int grid_max = sms * (per > 0 ? per : 1);
    const int g = n_jobs < grid_max ? n_jobs : grid_max;
    stage_tma<C><<<g, C::NT, smem, st>>>(a, n_jobs);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_tma_t() {
    int dev, optin;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return cudaFuncSetAttribute(stage_tma<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <class C>
StageVariant make_tma_variant(const char* name) {
    StageVariant v;
    v.L = C::L; v.CS = C::CS; v.NT = C::NT; v.smem = 0; v.np = C::NP;
    v.r[0] = C::R0; v.r[1] = C::R1; v.r[2] = C::R2; v.r[3] = C::R3;
    v.persistent = false;
    v.pipe = false;
    v.bf16 = false;
    v.tma = true;
    v.ctw = C::CTW;
    v.launch = &launch_tma_t<C>;
    v.prepare = &prepare_tma_t<C>;
    v.smem_for = &tma_smem<C>;
    v.name = name;
    return v;
}

}  // namespace pstd
