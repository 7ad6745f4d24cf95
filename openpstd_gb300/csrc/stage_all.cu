// stage_all.cu -- one persistent launch per RK stage over the strip jobs of
// every transform length 128 .. 2048 (all scenes of a batch or serving set).
//
// Per-length launches leave partial last waves: with three CTAs per SM a
// bucket of 928 jobs runs two full waves and a third of 16 CTAs, and every
// bucket ends on its own tail.  Here CTAs stay resident and take jobs from a
// per-stage counter (one atomicAdd per job; the jobs are ordered longest
// transform first), so the stage ends when the last job does.  Every length
// has a fixed configuration with one thread count, so all of them share one
// launch.  The counter is
// only read and incremented: when it passes the job count every CTA leaves.
// Two configuration families are compiled (MergedFam0 / MergedFam1 below).
//
// The job count is either a launch argument or read from device memory at the
// start of the launch (the serving loop: a captured graph keeps its grid and
// arguments while the job tables and their counts change in place between
// launches).  The serving loop keeps two tables in one array -- jobs of
// transform length >= 1024 first, the rest after a gap -- so that the long
// jobs are taken first; its free table entries are zero (length 0, no copy
// flag) and skipped, and so are the jobs of scenes that have taken all their
// steps.
#include <cstdlib>

#include "stage_kernel.cuh"

namespace pstd {

// Configuration families of the merged launch: per length the strips per job
// and radix plan, with one thread count and occupancy for all lengths (one
// launch), shared memory sized for the family's largest configuration.
// Family 0: 256 threads, 3 CTAs per SM, up to 66 KB per CTA (four complex
// strips of 2048).  Family 1: 128 threads, 8 CTAs per SM, 16.5 KB per CTA at
// every length (fewer strips per job as the length grows) and twiddle powers
// computed from a short table (the "ctw" form).
struct MergedFam0 {
    static constexpr int NT = 256, MINB = 3;
    using M128 = Cfg<128, 16, 256, 3, 16, 8>;
    using M256 = Cfg<256, 16, 256, 3, 16, 16>;
    using M512 = Cfg<512, 8, 256, 3, 8, 8, 8>;
    using M1024 = Cfg<1024, 8, 256, 3, 16, 8, 8>;
    using M2048 = Cfg<2048, 4, 256, 3, 16, 16, 8>;
};
struct MergedFam1 {
    static constexpr int NT = 128, MINB = 8;
    using M128 = Cfg<128, 16, 128, 8, 16, 8, 0, 0, 0, 0, 0, 1>;
    using M256 = Cfg<256, 8, 128, 8, 16, 16, 0, 0, 0, 0, 0, 1>;
    using M512 = Cfg<512, 4, 128, 8, 8, 8, 8, 0, 0, 0, 0, 1>;
    using M1024 = Cfg<1024, 2, 128, 8, 16, 8, 8, 0, 0, 0, 0, 1>;
    using M2048 = Cfg<2048, 1, 128, 8, 16, 16, 8, 0, 0, 0, 0, 1>;
};

template <class F>
constexpr int fam_smem() {
    constexpr int a = F::M128::SMEM > F::M256::SMEM ? F::M128::SMEM : F::M256::SMEM;
    constexpr int b = F::M512::SMEM > F::M1024::SMEM ? F::M512::SMEM : F::M1024::SMEM;
    constexpr int c = a > b ? a : b;
    return c > F::M2048::SMEM ? c : F::M2048::SMEM;
}
static_assert(fam_smem<MergedFam1>() <= 17 * 1024, "family 1 keeps 8 CTAs per SM");

// one strip job: the plain stage kernel's steps with the job's own twiddle table
// (not inlined: every length keeps its own register allocation; one call per
// job.  Inlined into the kernel's switch the five lengths spill 2.1 KB.)
template <class C, int NT>
__device__ __noinline__ void merged_job(float2* sm, const StageArgs& A, int j, int tid) {
    const DevJob job = A.jobs[j];
    const DevDomain dom = A.doms[job.dom];
    const bool first = A.first_step[dom.scene] != 0;
    gather<C, NT, false>(sm, A, job, dom, first, tid);
    __syncthreads();
    const bool vel = job.kind & JK_VEL;
    const int n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int nout = vel ? n - 1 : n + 1;
    convolve<C, NT, 0, false, true>(sm, A.tw + job.ttab, A.filt + job.dtab, tid, 2 * job.W + n, job.W, job.W + nout);
    __syncthreads();
    epilogue<C, NT>(sm, A, job, dom, tid);
}

// (the arguments stay in parameter space: the job functions read them by address)
template <class F>
__global__ void __launch_bounds__(F::NT, F::MINB) stage_all(const __grid_constant__ StageArgs A, int n_arg,
                                                            const int* counts, int* counter) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ int s_job;
    const int tid = threadIdx.x;
    int n_jobs = n_arg, n_first = n_arg, gap = 0;
    if (counts) {
        n_first = counts[0];
        n_jobs = n_first + counts[1];
        gap = counts[2] - n_first;   // the second table starts at counts[2]
    }
    for (;;) {
        if (tid == 0) s_job = atomicAdd(counter, 1);
        __syncthreads();
        int j = s_job;
        if (j >= n_jobs) break;   // the same value for the whole CTA
        if (j >= n_first) j += gap;
        const int kind = A.jobs[j].kind, L = A.jobs[j].L;
        bool live = true;
        if (A.scene_limit) {
            const int sc = A.doms[A.jobs[j].dom].scene;
            live = A.scene_step[sc] < A.scene_limit[sc];
        }
        if (!live) {
        } else if (kind & JK_COPY) {
            copy_axis<F::NT>(A, A.doms[A.jobs[j].dom], kind & JK_Y, tid);
        } else {
            switch (L) {
                case 128: merged_job<typename F::M128, F::NT>(sm, A, j, tid); break;
                case 256: merged_job<typename F::M256, F::NT>(sm, A, j, tid); break;
                case 512: merged_job<typename F::M512, F::NT>(sm, A, j, tid); break;
                case 1024: merged_job<typename F::M1024, F::NT>(sm, A, j, tid); break;
                case 2048: merged_job<typename F::M2048, F::NT>(sm, A, j, tid); break;
                default: break;
            }
        }
        __syncthreads();   // shared memory and s_job are reused by the next job
    }
}

bool merged_supports(int L) { return L == 128 || L == 256 || L == 512 || L == 1024 || L == 2048; }

int merged_family_default() {
    if (const char* e = std::getenv("PSTD_MERGED_FAMILY")) return std::atoi(e) == 1 ? 1 : 0;
    return 1;
}

// the configuration family `fam` uses for L (strips per job and radix plan
// for the job lists and tables)
const StageVariant* merged_variant(int L, int fam) {
    static const StageVariant v0[] = {
        make_variant<MergedFam0::M128>("L128 cs16 nt256 r16.8 (merged)"),
        make_variant<MergedFam0::M256>("L256 cs16 nt256 r16.16 (merged)"),
        make_variant<MergedFam0::M512>("L512 cs8 nt256 r8.8.8 (merged)"),
        make_variant<MergedFam0::M1024>("L1024 cs8 nt256 r16.8.8 (merged)"),
        make_variant<MergedFam0::M2048>("L2048 cs4 nt256 r16.16.8 (merged)"),
    };
    static const StageVariant v1[] = {
        make_variant<MergedFam1::M128>("L128 cs16 nt128 mb8 r16.8 ctw (merged)"),
        make_variant<MergedFam1::M256>("L256 cs8 nt128 mb8 r16.16 ctw (merged)"),
        make_variant<MergedFam1::M512>("L512 cs4 nt128 mb8 r8.8.8 ctw (merged)"),
        make_variant<MergedFam1::M1024>("L1024 cs2 nt128 mb8 r16.8.8 ctw (merged)"),
        make_variant<MergedFam1::M2048>("L2048 cs1 nt128 mb8 r16.16.8 ctw (merged)"),
    };
    const StageVariant* v = fam == 1 ? v1 : v0;
    switch (L) {
        case 128: return &v[0];
        case 256: return &v[1];
        case 512: return &v[2];
        case 1024: return &v[3];
        case 2048: return &v[4];
        default: return nullptr;
    }
}

template <class F>
static cudaError_t prepare_fam() {
    return cudaFuncSetAttribute(stage_all<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, fam_smem<F>());
}

cudaError_t prepare_stage_all(int fam) { return fam == 1 ? prepare_fam<MergedFam1>() : prepare_fam<MergedFam0>(); }

// resident CTAs of the merged launch on this device (SMs x CTAs per SM)
template <class F>
static int stage_all_grid() {
    static int grid = 0;
    if (grid == 0) {
        int dev, sms, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stage_all<F>, F::NT, fam_smem<F>());
        grid = sms * (per > 0 ? per : 1);
    }
    return grid;
}

template <class F>
static cudaError_t launch_fam(int n_jobs, const int* counts, const StageArgs& a, int* counter, cudaStream_t st) {
    int g = stage_all_grid<F>();
    if (!counts) {
        if (n_jobs <= 0) return cudaSuccess;
        g = n_jobs < g ? n_jobs : g;
    }
    stage_all<F><<<g, F::NT, fam_smem<F>(), st>>>(a, n_jobs, counts, counter);
    return cudaGetLastError();
}

cudaError_t launch_stage_all(int fam, int n_jobs, const StageArgs& a, int* counter, cudaStream_t st) {
    return fam == 1 ? launch_fam<MergedFam1>(n_jobs, nullptr, a, counter, st)
                    : launch_fam<MergedFam0>(n_jobs, nullptr, a, counter, st);
}

cudaError_t launch_stage_all_dev(int fam, const int* counts, const StageArgs& a, int* counter, cudaStream_t st) {
    return fam == 1 ? launch_fam<MergedFam1>(0, counts, a, counter, st)
                    : launch_fam<MergedFam0>(0, counts, a, counter, st);
}

}  // namespace pstd
