// stage_all.cu -- one persistent launch per RK stage over the strip jobs of
// every transform length 128 .. 2048 (all scenes of a batch or serving set).
//
// Per-length launches leave partial last waves: with three CTAs per SM a
// bucket of 928 jobs runs two full waves and a third of 16 CTAs, and every
// bucket ends on its own tail.  Here CTAs stay resident and take jobs from a
// per-stage counter (one atomicAdd per job; the jobs are ordered longest
// transform first), so the stage ends when the last job does.  Every length
// has a fixed configuration with 256 threads and at most 66 KB of shared
// memory, so all of them share one launch (3 CTAs per SM).  The counter is
// only read and incremented: when it passes the job count every CTA leaves.
#include "stage_kernel.cuh"

namespace pstd {

// per-length configurations of the merged launch (strips per job, radix plan)
using M128 = Cfg<128, 16, 256, 3, 16, 8>;
using M256 = Cfg<256, 16, 256, 3, 16, 16>;
using M512 = Cfg<512, 8, 256, 3, 8, 8, 8>;
using M1024 = Cfg<1024, 8, 256, 3, 16, 8, 8>;
using M2048 = Cfg<2048, 4, 256, 3, 16, 16, 8>;

constexpr int MERGED_NT = 256;
constexpr int MERGED_SMEM = M2048::SMEM > M1024::SMEM ? M2048::SMEM : M1024::SMEM;
static_assert(M128::SMEM <= MERGED_SMEM && M256::SMEM <= MERGED_SMEM && M512::SMEM <= MERGED_SMEM,
              "the merged launch sizes shared memory for its largest configuration");

// one strip job: the plain stage kernel's steps with the job's own twiddle table
// (not inlined: every length keeps its own register allocation; one call per job)
template <class C>
__device__ __noinline__ void merged_job(float2* sm, const StageArgs& A, int j, int tid) {
    const DevJob job = A.jobs[j];
    const DevDomain dom = A.doms[job.dom];
    const bool first = A.first_step[dom.scene] != 0;
    gather<C, MERGED_NT, false>(sm, A, job, dom, first, tid);
    __syncthreads();
    const bool vel = job.kind & JK_VEL;
    const int n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int nout = vel ? n - 1 : n + 1;
    convolve<C, MERGED_NT, 0, false, true>(sm, A.tw + job.ttab, A.filt + job.dtab, tid, 2 * job.W + n, job.W,
                                           job.W + nout);
    __syncthreads();
    epilogue<C, MERGED_NT>(sm, A, job, dom, tid);
}

// (the arguments stay in parameter space: the job functions read them by address)
__global__ void __launch_bounds__(MERGED_NT, 3) stage_all(const __grid_constant__ StageArgs A, int n_jobs, int* counter) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ int s_job;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_job = atomicAdd(counter, 1);
        __syncthreads();
        const int j = s_job;
        if (j >= n_jobs) break;   // the same value for the whole CTA
        const int kind = A.jobs[j].kind, L = A.jobs[j].L;
        if (kind & JK_COPY) {
            copy_axis<MERGED_NT>(A, A.doms[A.jobs[j].dom], kind & JK_Y, tid);
        } else {
            switch (L) {
                case 128: merged_job<M128>(sm, A, j, tid); break;
                case 256: merged_job<M256>(sm, A, j, tid); break;
                case 512: merged_job<M512>(sm, A, j, tid); break;
                case 1024: merged_job<M1024>(sm, A, j, tid); break;
                case 2048: merged_job<M2048>(sm, A, j, tid); break;
                default: break;
            }
        }
        __syncthreads();   // shared memory and s_job are reused by the next job
    }
}

bool merged_supports(int L) { return L == 128 || L == 256 || L == 512 || L == 1024 || L == 2048; }

// the configuration the merged launch uses for L (strips per job and radix
// plan for the job lists and tables)
const StageVariant* merged_variant(int L) {
    static const StageVariant v[] = {
        make_variant<M128>("L128 cs16 nt256 r16.8 (merged)"),
        make_variant<M256>("L256 cs16 nt256 r16.16 (merged)"),
        make_variant<M512>("L512 cs8 nt256 r8.8.8 (merged)"),
        make_variant<M1024>("L1024 cs8 nt256 r16.8.8 (merged)"),
        make_variant<M2048>("L2048 cs4 nt256 r16.16.8 (merged)"),
    };
    switch (L) {
        case 128: return &v[0];
        case 256: return &v[1];
        case 512: return &v[2];
        case 1024: return &v[3];
        case 2048: return &v[4];
        default: return nullptr;
    }
}

cudaError_t prepare_stage_all() {
    return cudaFuncSetAttribute(stage_all, cudaFuncAttributeMaxDynamicSharedMemorySize, MERGED_SMEM);
}

cudaError_t launch_stage_all(int n_jobs, const StageArgs& a, int* counter, cudaStream_t st) {
    if (n_jobs <= 0) return cudaSuccess;
    static int grid = 0;
    if (grid == 0) {
        int dev, sms, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stage_all, MERGED_NT, MERGED_SMEM);
        grid = sms * (per > 0 ? per : 1);
    }
    const int g = n_jobs < grid ? n_jobs : grid;
    stage_all<<<g, MERGED_NT, MERGED_SMEM, st>>>(a, n_jobs, counter);
    return cudaGetLastError();
}

}  // namespace pstd
