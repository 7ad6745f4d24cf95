// stage_toeplitz.cu -- the L = 128 strips' derivative as a tcgen05 GEMM.
//
// The transform pair of a strip is a circular convolution with the real
// kernel h of the derivative factors (stage_direct.cu): for the outputs at
// buf positions W + c,
//   out[W + c] = sum_j buf[j] h[(W + c - j) mod L],
// i.e. one row of strips times a Toeplitz matrix.  One CTA takes a job of up
// to 128 strips (the GEMM's M) and computes
//   D (128 strips x 80 outputs) = A (128 x K = 128 inputs) * B (128 x 80)
// on the tensor core, kind::tf32 with FP32 accumulation in TMEM, operands
// split three ways (x = x_hi + x_lo, TF32 each; hi*hi, and hi*lo + lo*hi in a
// second accumulator, the lo*lo term dropped: about 2^-21 relative).
//
// B is Toeplitz, so all sixteen K = 8 slices of it are windows of one
// extended tile E (200 rows x 8 inputs): slice kb (inputs 8kb .. 8kb+7) is E's
// rows 120 - 8kb .. 199 - 8kb, E[r][u] = h[(W + r - 120 - u) mod L], and the
// slice's descriptor only moves its start address by whole 8-row groups.
// The strips are gathered by the plain form's gather (bands, reflection /
// transmission, window, zero padding), converted to the A tiles, and the
// results go back through shared memory to the plain form's epilogue (RK
// update, PML on vx / vy at the sixth stage).  Shared-memory operand layout:
// K-major, no swizzle (8-row x 16-byte core matrices).
//
// The one thread that issues the MMAs commits them to an mbarrier; the
// wait is bounded: on a timeout the CTA records error 2 in *A.err, waits once
// more (bounded) for its MMAs, frees its TMEM and leaves.  A job outside the
// form's fixed tile (window 32, n + 2W <= 128, at most 80 outputs) records
// error 3 and is not computed; the L = 128 bucket never has one (its strips
// have n in 32..63 and W = 32).
#include "stage_tc5.cuh"

namespace pstd {

namespace toe {
constexpr int L = 128, W = 32, ROWS = 128, K = 128, N = 80;
constexpr int EROWS = N + K - 8;            // rows of the extended kernel tile
constexpr int A_WORDS = ROWS * K;           // one A tile (64 KB)
constexpr int E_WORDS = EROWS * 8;          // one E tile (6.4 KB)
constexpr uint32_t A_LBO = 128, A_SBO = (K / 4) * 128;   // core matrices along K / along M
constexpr uint32_t E_LBO = 128, E_SBO = 256;             // along K / along N
constexpr int D1_COL = 128;                 // cross-term accumulator
constexpr int TMEM_COLS = 256;
}  // namespace toe

// word offsets in the operand tiles (K-major, no swizzle)
__device__ __forceinline__ int toe_a_off(int row, int k) {
    return (row >> 3) * (toe::K / 4 * 32) + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}
__device__ __forceinline__ int toe_e_off(int r, int u) {
    return (r >> 3) * 64 + (u >> 2) * 32 + (r & 7) * 4 + (u & 3);
}

// 8 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

template <class C>
constexpr size_t toe_smem() {
    return (size_t)C::BUF * 8 + 128 + (size_t)(2 * toe::A_WORDS + 2 * toe::E_WORDS) * 4 + 16;
}

template <class C>
__global__ void __launch_bounds__(C::NT, 1) stage_toe(StageArgs A) {
    static_assert(C::L == toe::L && 2 * C::CS == toe::ROWS, "one 128-strip GEMM per job");
    static_assert(C::NT == 256, "warps 0-3 and 4-7 read the two column halves of the accumulators");
    extern __shared__ __align__(16) float2 sm[];
    constexpr int NT = C::NT;
    // strips, then (128-byte aligned) A_hi, A_lo, E_hi, E_lo, mbarrier, TMEM address
    unsigned char* base = reinterpret_cast<unsigned char*>(sm) + (size_t)C::BUF * 8;
    base += (128u - (smem_addr(base) & 127u)) & 127u;
    uint32_t* a_hi = reinterpret_cast<uint32_t*>(base);
    uint32_t* a_lo = a_hi + toe::A_WORDS;
    uint32_t* e_hi = a_lo + toe::A_WORDS;
    uint32_t* e_lo = e_hi + toe::E_WORDS;
    uint64_t* bar = reinterpret_cast<uint64_t*>(e_lo + toe::E_WORDS);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    if (job.kind & JK_COPY) {
        copy_axis<NT>(A, dom, job.kind & JK_Y, tid);
        return;
    }
    const bool vel = job.kind & JK_VEL;
    const int n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int nout = vel ? n - 1 : n + 1;
    if (job.W != toe::W || 2 * job.W + n > toe::K || nout > toe::N || job.count > toe::ROWS) {
        if (tid == 0 && A.err) atomicExch(A.err, 3);
        return;
    }
    // E[r][u] = h[(W + r - (K - 8) - u) mod L] from the extended table hx[e] = h[(e - L) mod L]
    const float* hx = reinterpret_cast<const float*>(A.filt + job.dtab);
    for (int i = tid; i < toe::E_WORDS; i += NT) {
        const int r = i >> 3, u = i & 7;
        const float v = hx[toe::W + r - (toe::K - 8) - u + toe::L];
        const uint32_t hi = f32_to_tf32(v);
        e_hi[toe_e_off(r, u)] = hi;
        e_lo[toe_e_off(r, u)] = f32_to_tf32(v - __uint_as_float(hi));
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "n"(toe::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const bool first = A.first_step[dom.scene] != 0;
    gather<C, NT, true>(sm, A, job, dom, first, tid);
    __syncthreads();
    // strips -> A rows, TF32 hi / lo; a warp covers 8 rows x 4 inputs (distinct banks in the tiles)
    {
        const float* smf = reinterpret_cast<const float*>(sm);
        for (int i = tid; i < toe::ROWS * toe::K; i += NT) {
            const int sub = i & 31, blk = i >> 5;
            const int row = (blk % (toe::ROWS / 8)) * 8 + (sub & 7);
            const int k = (blk / (toe::ROWS / 8)) * 4 + (sub >> 3);
            const float v = smf[2 * ((row >> 1) * C::SP + k) + (row & 1)];
            const uint32_t hi = f32_to_tf32(v);
            a_hi[toe_a_off(row, k)] = hi;
            a_lo[toe_a_off(row, k)] = f32_to_tf32(v - __uint_as_float(hi));
        }
    }
    fence_async_smem();   // the tiles written by this CTA's threads, seen by the tensor core
    __syncthreads();
    if (tid == 0) {
        tc_fence_after();
        constexpr uint32_t idesc = umma_idesc_tf32(toe::ROWS, toe::N);
#pragma unroll
        for (int kb = 0; kb < toe::K / 8; kb++) {   // K = 8 per instruction: two core matrices
            const uint64_t ah = umma_desc(a_hi + kb * 64, toe::A_LBO, toe::A_SBO);
            const uint64_t al = umma_desc(a_lo + kb * 64, toe::A_LBO, toe::A_SBO);
            const int g = toe::K / 8 - 1 - kb;      // E's 8-row group where slice kb starts
            const uint64_t bh = umma_desc(e_hi + g * 64, toe::E_LBO, toe::E_SBO);
            const uint64_t bl = umma_desc(e_lo + g * 64, toe::E_LBO, toe::E_SBO);
            const uint32_t acc = kb > 0 ? 1u : 0u;
            umma_tf32(tmem + toe::D1_COL, al, bh, idesc, acc);
            umma_tf32(tmem + toe::D1_COL, ah, bl, idesc, 1);
            umma_tf32(tmem, ah, bh, idesc, acc);
        }
        umma_commit(bar);
    }
    const bool ok = __syncthreads_and(mbar_wait(bar, 0)) != 0;
    tc_fence_after();
    if (ok) {
        // warp w reads lanes 32 (w % 4) .. (its 32 strips), columns [40 (w / 4), 40 (w / 4) + 40)
        const int s = 32 * (warp & 3) + lane;
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        float* smw = reinterpret_cast<float*>(sm);
        const int c_lo = (warp >> 2) * (toe::N / 2);
#pragma unroll
        for (int c0 = c_lo; c0 < c_lo + toe::N / 2; c0 += 8) {
            float big[8], small[8];
            tmem_ld8(tmem + lane_base + (uint32_t)c0, big);
            tmem_ld8(tmem + lane_base + (uint32_t)(toe::D1_COL + c0), small);
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (c0 + q < nout) smw[2 * ((s >> 1) * C::SP + toe::W + c0 + q) + (s & 1)] = small[q] + big[q];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (ok) {
        epilogue<C, NT>(sm, A, job, dom, tid);
    } else if (tid == 0) {
        if (A.err) atomicExch(A.err, 2);
        mbar_wait(bar, 0);   // bounded: the MMAs, before their TMEM is freed
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(toe::TMEM_COLS)
                     : "memory");
}

template <class C>
cudaError_t launch_toe_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    if (n_jobs <= 0) return cudaSuccess;
    stage_toe<C><<<n_jobs, C::NT, toe_smem<C>(), st>>>(a);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_toe_t() {
    return cudaFuncSetAttribute(stage_toe<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)toe_smem<C>());
}

template <class C>
size_t toe_smem_for(int) {
    return toe_smem<C>();
}

template <class C>
StageVariant make_toe_variant(const char* name) {
    StageVariant v = make_variant<C>(name);
    v.smem = (int)toe_smem<C>();
    v.direct = 8;   // the kernel table of the direct forms (hx, 2L + 8 floats)
    v.launch = &launch_toe_t<C>;
    v.prepare = &prepare_toe_t<C>;
    v.smem_for = &toe_smem_for<C>;
    return v;
}

const StageVariant* stage_variants_toeplitz(int L, int* n) {
    static const StageVariant v128[] = {
        make_toe_variant<Cfg<128, 64, 256, 1, 16, 8>>("L128 cs64 nt256 tcgen05 toeplitz tf32x3"),
    };
    switch (L) {
        case 128: *n = 1; return v128;
        default: *n = 0; return nullptr;
    }
}



// ---------------------------------------------------------------- persistent, warp-specialised form
// One CTA per SM walks its share of the jobs (job = blockIdx.x + t * gridDim.x)
// with three roles running on different jobs at once:
//   warps 4-11 (producers) gather job t into the strip buffer (the plain
//     form's gather), then -- once the tensor core is done with job t-1's
//     operands -- split it into the A tiles, build E and hand the stage over;
//   warp 12 (one thread) issues job t's 48 MMAs into TMEM accumulator pair
//     t % 2 (once the epilogue has emptied it) and commits them;
//   warps 0-3 (epilogue) read job t-1's accumulators (lanes = strips),
//     free them, and apply the RK update (rows through a small per-warp
//     staging tile, so that a warp writes 4 rows x 8 outputs per store).
// Hand-overs are mbarriers: a_full (producers -> MMA), a_free (MMA commit ->
// producers), d_full[2] (MMA commit -> epilogue), d_free[2] (epilogue -> MMA).
// Every wait is bounded; a role that gives up records error 2 and leaves its
// loop, the others give up at their next wait, and the MMA thread waits
// (bounded) for its last commit before the TMEM is freed.
namespace toews {
constexpr int EPI_WARPS = 4, PROD_WARPS = 8;
constexpr int NT = 32 * (EPI_WARPS + PROD_WARPS + 1);
constexpr int PROD0 = 32 * EPI_WARPS, NPROD = 32 * PROD_WARPS, MMA_WARP = EPI_WARPS + PROD_WARPS;
constexpr int STG = 9;             // staging pitch (floats): a warp's 32 strips x 8 outputs
constexpr int TMEM_COLS = 512;     // two accumulator pairs of 256 columns
constexpr int BAR_PROD = 1;        // named barrier of the producers
}  // namespace toews

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// the job fits the form's fixed tile (otherwise error 3, not computed)
__device__ __forceinline__ bool toe_fits(const DevJob& job, const DevDomain& dom, int& n, int& nout) {
    const bool vel = job.kind & JK_VEL;
    n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
    nout = vel ? n - 1 : n + 1;
    return job.W == toe::W && 2 * job.W + n <= toe::K && nout <= toe::N && job.count <= toe::ROWS;
}

template <class C>
constexpr size_t toews_smem() {
    return (size_t)C::BUF * 8 + 128 + (size_t)(2 * toe::A_WORDS + 2 * toe::E_WORDS) * 4 +
           (size_t)toews::EPI_WARPS * 32 * toews::STG * 4 + 6 * 8 + 16;
}

template <class C>
__global__ void __launch_bounds__(toews::NT, 1) stage_toe_ws(StageArgs A, int n_jobs) {
    static_assert(C::L == toe::L && 2 * C::CS == toe::ROWS && C::NT == toews::NT, "one 128-strip GEMM per job");
    extern __shared__ __align__(16) float2 sm[];
    using namespace toews;
    float2* buf = sm;
    unsigned char* base = reinterpret_cast<unsigned char*>(sm) + (size_t)C::BUF * 8;
    base += (128u - (smem_addr(base) & 127u)) & 127u;
    uint32_t* a_hi = reinterpret_cast<uint32_t*>(base);
    uint32_t* a_lo = a_hi + toe::A_WORDS;
    uint32_t* e_hi = a_lo + toe::A_WORDS;
    uint32_t* e_lo = e_hi + toe::E_WORDS;
    float* stg = reinterpret_cast<float*>(e_lo + toe::E_WORDS);
    uint64_t* bars = reinterpret_cast<uint64_t*>(stg + EPI_WARPS * 32 * STG);
    uint64_t* a_full = bars;
    uint64_t* a_free = bars + 1;
    uint64_t* d_full = bars + 2;   // [2]
    uint64_t* d_free = bars + 4;   // [2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 6);
    int* pfail = reinterpret_cast<int*>(tslot + 1);   // producers' shared give-up flag
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        mbar_init(a_full, 1);
        mbar_init(a_free, 1);
        mbar_init(d_full, 1);
        mbar_init(d_full + 1, 1);
        mbar_init(d_free, EPI_WARPS);
        mbar_init(d_free + 1, EPI_WARPS);
        *pfail = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "n"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp >= EPI_WARPS && warp < MMA_WARP) {
        // ---- producers
        const int ptid = tid - PROD0;
        int g = 0;
        for (int j = blockIdx.x; j < n_jobs; j += gridDim.x) {
            const DevJob job = A.jobs[j];
            const DevDomain dom = A.doms[job.dom];
            if (job.kind & JK_COPY) {
                copy_axis<NPROD>(A, dom, job.kind & JK_Y, ptid);
                continue;
            }
            int n, nout;
            if (!toe_fits(job, dom, n, nout)) {
                if (ptid == 0 && A.err) atomicExch(A.err, 3);
                continue;
            }
            const bool first = A.first_step[dom.scene] != 0;
            gather<C, NPROD, true>(buf, A, job, dom, first, ptid);
            if (ptid == 0 && g > 0 && !mbar_wait(a_free, (g - 1) & 1)) *pfail = 1;   // job g-1's operands read
            bar_sync(BAR_PROD, NPROD);
            if (*pfail) break;
            // E[r][u] = h[(W + r - (K - 8) - u) mod L]
            const float* hx = reinterpret_cast<const float*>(A.filt + job.dtab);
            for (int i = ptid; i < toe::E_WORDS; i += NPROD) {
                const int r = i >> 3, u = i & 7;
                const float v = hx[toe::W + r - (toe::K - 8) - u + toe::L];
                const uint32_t hi = f32_to_tf32(v);
                e_hi[toe_e_off(r, u)] = hi;
                e_lo[toe_e_off(r, u)] = f32_to_tf32(v - __uint_as_float(hi));
            }
            const float* smf = reinterpret_cast<const float*>(buf);
            for (int i = ptid; i < toe::ROWS * toe::K; i += NPROD) {
                const int sub = i & 31, blk = i >> 5;
                const int row = (blk % (toe::ROWS / 8)) * 8 + (sub & 7);
                const int k = (blk / (toe::ROWS / 8)) * 4 + (sub >> 3);
                const float v = smf[2 * ((row >> 1) * C::SP + k) + (row & 1)];
                const uint32_t hi = f32_to_tf32(v);
                a_hi[toe_a_off(row, k)] = hi;
                a_lo[toe_a_off(row, k)] = f32_to_tf32(v - __uint_as_float(hi));
            }
            fence_async_smem();   // this thread's tile writes, for the tensor core
            bar_sync(BAR_PROD, NPROD);   // all tiles written; the strip buffer is free again
            if (ptid == 0) mbar_arrive(a_full);
            ++g;
        }
    } else if (warp == MMA_WARP) {
        // ---- MMA issue (one thread)
        if (lane == 0) {
            int g = 0;
            bool ok = true;
            for (int j = blockIdx.x; j < n_jobs && ok; j += gridDim.x) {
                const DevJob job = A.jobs[j];
                const DevDomain dom = A.doms[job.dom];
                int n, nout;
                if ((job.kind & JK_COPY) || !toe_fits(job, dom, n, nout)) continue;
                const int b = g & 1;
                ok = mbar_wait(a_full, g & 1) && (g < 2 || mbar_wait(d_free + b, ((g - 2) >> 1) & 1));
                if (!ok) break;
                tc_fence_after();
                constexpr uint32_t idesc = umma_idesc_tf32(toe::ROWS, toe::N);
                const uint32_t d0 = tmem + (uint32_t)(b * 256), d1 = d0 + toe::D1_COL;
#pragma unroll
                for (int kb = 0; kb < toe::K / 8; kb++) {
                    const uint64_t ah = umma_desc(a_hi + kb * 64, toe::A_LBO, toe::A_SBO);
                    const uint64_t al = umma_desc(a_lo + kb * 64, toe::A_LBO, toe::A_SBO);
                    const int eg = toe::K / 8 - 1 - kb;
                    const uint64_t bh = umma_desc(e_hi + eg * 64, toe::E_LBO, toe::E_SBO);
                    const uint64_t bl = umma_desc(e_lo + eg * 64, toe::E_LBO, toe::E_SBO);
                    const uint32_t acc = kb > 0 ? 1u : 0u;
                    umma_tf32(d1, al, bh, idesc, acc);
                    umma_tf32(d1, ah, bl, idesc, 1);
                    umma_tf32(d0, ah, bh, idesc, acc);
                }
                umma_commit(a_free);
                umma_commit(d_full + b);
                ++g;
            }
            if (!ok && A.err) atomicExch(A.err, 2);
            if (g > 0) mbar_wait(d_full + ((g - 1) & 1), ((g - 1) >> 1) & 1);   // bounded: the last MMAs
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w holds strips 32 w .. 32 w + 31 (TMEM lanes)
        const int s = 32 * warp + lane;
        const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
        float* st = stg + warp * 32 * STG;
        int g = 0;
        for (int j = blockIdx.x; j < n_jobs; j += gridDim.x) {
            const DevJob job = A.jobs[j];
            const DevDomain dom = A.doms[job.dom];
            int n, nout;
            if ((job.kind & JK_COPY) || !toe_fits(job, dom, n, nout)) continue;
            const int b = g & 1;
            const bool ok = __all_sync(0xffffffffu, mbar_wait(d_full + b, (g >> 1) & 1));
            if (!ok) {
                if (lane == 0 && A.err) atomicExch(A.err, 2);
                break;
            }
            tc_fence_after();
            float d[toe::N];
            const uint32_t d0 = tmem + lane_base + (uint32_t)(b * 256);
#pragma unroll
            for (int c0 = 0; c0 < toe::N; c0 += 8) {
                float big[8], small[8];
                tmem_ld8(d0 + (uint32_t)c0, big);
                tmem_ld8(d0 + (uint32_t)(toe::D1_COL + c0), small);
#pragma unroll
                for (int q = 0; q < 8; q++) d[c0 + q] = small[q] + big[q];
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(d_free + b);   // the accumulators of job g are read
            // RK update (kernel/Solver.cpp:162-182), as the plain epilogue
            const bool vel = job.kind & JK_VEL, ydir = job.kind & JK_Y;
            long long fo;
            int fp, ao;
            if (!vel) { fo = ydir ? dom.o_vy : dom.o_vx; fp = ydir ? dom.pitch_vy : dom.pitch_vx; ao = ydir ? dom.att_yv : dom.att_xv; }
            else { fo = ydir ? dom.o_py : dom.o_px; fp = dom.pitch_p; ao = -1; }
            const bool att = !vel && A.last && ao >= 0;
            const float cdt = A.doms[job.dom].cdt[A.stage];
            const float rho = dom.rho, c2 = dom.c2, rinv = __frcp_rn(rho);
            const float* __restrict__ prev = A.prev;
            float* __restrict__ out = A.out;
            if (ydir) {
                // columns: consecutive lanes on consecutive columns
                if (s < job.count) {
#pragma unroll
                    for (int i = 0; i < toe::N; i++) {
                        if (i < nout) {
                            const long long e = fo + (long long)i * fp + job.first + s;
                            float v = rk_update(prev[e], d[i], vel, cdt, rho, c2, rinv);
                            if (att) v = __fmul_rn(v, A.att[ao + i]);
                            out[e] = v;
                        }
                    }
                }
            } else {
                // rows: through the staging tile, lanes 8r .. 8r+7 on 8 outputs of row r
#pragma unroll
                for (int c0 = 0; c0 < toe::N; c0 += 8) {
                    if (c0 >= nout) continue;   // warp-uniform
#pragma unroll
                    for (int q = 0; q < 8; q++) st[lane * STG + q] = d[c0 + q];
                    __syncwarp();
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const int r = 4 * k + (lane >> 3), q = lane & 7, i = c0 + q, sr = 32 * warp + r;
                        if (sr < job.count && i < nout) {
                            const long long e = fo + (long long)(job.first + sr) * fp + i;
                            float v = rk_update(prev[e], st[r * STG + q], vel, cdt, rho, c2, rinv);
                            if (att) v = __fmul_rn(v, A.att[ao + i]);
                            out[e] = v;
                        }
                    }
                    __syncwarp();
                }
            }
            ++g;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TMEM_COLS) : "memory");
}

template <class C>
cudaError_t launch_toews_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    if (n_jobs <= 0) return cudaSuccess;
    static int sms = 0;
    if (sms == 0) {
        int dev;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const int grid = n_jobs < sms ? n_jobs : sms;
    stage_toe_ws<C><<<grid, toews::NT, toews_smem<C>(), st>>>(a, n_jobs);
    return cudaGetLastError();
}

template <class C>
cudaError_t prepare_toews_t() {
    return cudaFuncSetAttribute(stage_toe_ws<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)toews_smem<C>());
}

template <class C>
size_t toews_smem_for(int) {
    return toews_smem<C>();
}

template <class C>
StageVariant make_toews_variant(const char* name) {
    StageVariant v = make_variant<C>(name);
    v.smem = (int)toews_smem<C>();
    v.direct = 8;
    v.launch = &launch_toews_t<C>;
    v.prepare = &prepare_toews_t<C>;
    v.smem_for = &toews_smem_for<C>;
    return v;
}

const StageVariant* stage_variants_toeplitz_ws(int L, int* n) {
    static const StageVariant v128[] = {
        make_toews_variant<Cfg<128, 64, toews::NT, 1, 16, 8>>("L128 cs64 ws416 tcgen05 toeplitz tf32x3"),
    };
    switch (L) {
        case 128: *n = 1; return v128;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
