// stage_direct.cu -- stage-kernel variants for short strips (L = 128) that
// apply the derivative as a direct circular convolution instead of a
// transform pair.
//
// spatderp3 (kernel/core/kernel_functions.cpp:123-318) computes, for the
// windowed strip buf (n + 2W values, zero-padded to L),
//   out[t] = c2r(r2c(buf) * derfact)[t] / L = sum_j buf[j] h[(t - j) mod L],
//   h[d]   = (1/L) sum_k D[k] exp(2 pi i k d / L),
// D the Hermitian extension of the derivative factors (the c2r drops the
// imaginary parts of the DC and Nyquist bins).  h is real, built in double on
// the host and rounded once to float.  For the PML-normal strips of the
// L = 128 bucket (n <= 64: about 51 outputs from 114 inputs) the sum is a few
// thousand FMAs per strip with no barrier between passes, against two
// forward and two inverse radix passes with a barrier after each.  The
// gather (bands, reflection / transmission, window) and the epilogue (RK
// update, PML on vx / vy at the sixth stage) are the plain form's.
//
// Shared memory: the gathered strips (CS complex strips: two real strips as
// re / im, as the transform forms keep them), the outputs in the same layout,
// and the kernel extended to 2L + Q floats, hx[e] = h[(e - L) mod L], so that
// every (t - j) + L + m below lies inside it without a modulo.
#include "stage_kernel.cuh"

namespace pstd {

// out[s][t] for t in [lo, hi), every complex strip s < CS; inputs [0, z0)
// (zero from z0 to L: the gather zero-fills).  One task = Q consecutive
// outputs of one strip; inputs are taken Q at a time, with the 2Q - 1 kernel
// values that block of outputs and inputs needs held in registers.  Threads
// of a warp take the same output block of different strips: the kernel
// values are a broadcast, the strips' inputs fall in distinct bank pairs
// (strip pitch Cfg::SP).
template <class C, int NTH, int Q>
__device__ __forceinline__ void direct_conv(const float2* __restrict__ in, float2* __restrict__ out,
                                            const float* __restrict__ hx, int tid, int z0, int lo, int hi) {
    constexpr int CS = C::CS, SP = C::SP, L = C::L;
    static_assert(L % Q == 0, "outputs and inputs are taken in blocks of Q");
    const int nb = (hi - lo + Q - 1) / Q;
    const int jn = (z0 + Q - 1) / Q;   // <= L / Q: blocks end inside the zero-filled strip
    for (int t = tid; t < CS * nb; t += NTH) {
        const int s = t % CS, b = t / CS;
        const int i0 = lo + b * Q;
        const float2* x = in + s * SP;
        float2 acc[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) acc[q] = make_float2(0.f, 0.f);
        // hw[m] = h[(i0 + m - (Q - 1) - j0) mod L] = hx[i0 - j0 + L - (Q - 1) + m], m < 2Q - 1
        const float* hb = hx + i0 + L - (Q - 1);
        for (int jb = 0; jb < jn; jb++) {
            const int j0 = jb * Q;
            float hw[2 * Q - 1];
#pragma unroll
            for (int m = 0; m < 2 * Q - 1; m++) hw[m] = hb[m - j0];
#pragma unroll
            for (int u = 0; u < Q; u++) {
                const float2 v = x[j0 + u];
#pragma unroll
                for (int q = 0; q < Q; q++) {   // output i0 + q, input j0 + u: h[(i0 + q - j0 - u) mod L]
                    const float hv = hw[q - u + Q - 1];
                    acc[q].x = fmaf(hv, v.x, acc[q].x);
                    acc[q].y = fmaf(hv, v.y, acc[q].y);
                }
            }
        }
        float2* o = out + s * SP;
#pragma unroll
        for (int q = 0; q < Q; q++)
            if (i0 + q < hi) o[i0 + q] = acc[q];
    }
}

template <class C, int Q>
__global__ void __launch_bounds__(C::NT, C::MINB) stage_direct(StageArgs A) {
    extern __shared__ __align__(16) float2 sm[];
    const DevJob job = A.jobs[blockIdx.x];
    const DevDomain dom = A.doms[job.dom];
    if (job.kind & JK_COPY) {
        copy_axis<C::NT>(A, dom, job.kind & JK_Y, threadIdx.x);
        return;
    }
    float2* res = sm + C::BUF;
    float* hx = reinterpret_cast<float*>(sm + 2 * C::BUF);
    const float* hsrc = reinterpret_cast<const float*>(A.filt + job.dtab);
    for (int e = threadIdx.x; e < 2 * C::L + Q; e += C::NT) hx[e] = hsrc[e];
    const bool first = A.first_step[dom.scene] != 0;
    gather<C, C::NT, true>(sm, A, job, dom, first, threadIdx.x);
    __syncthreads();
    const bool vel = job.kind & JK_VEL;
    const int n = ((job.kind & JK_Y) ? dom.ny : dom.nx) + (vel ? 1 : 0);
    const int nout = vel ? n - 1 : n + 1;
    direct_conv<C, C::NT, Q>(sm, res, hx, threadIdx.x, 2 * job.W + n, job.W, job.W + nout);
    __syncthreads();
    epilogue<C, C::NT>(res, A, job, dom, threadIdx.x);
}

template <class C, int Q>
constexpr size_t direct_smem() {
    return (size_t)2 * C::BUF * sizeof(float2) + (size_t)(2 * C::L + Q) * sizeof(float);
}

template <class C, int Q>
size_t direct_smem_for(int) {
    return direct_smem<C, Q>();
}

template <class C, int Q>
cudaError_t launch_direct_t(int n_jobs, const StageArgs& a, cudaStream_t st) {
    if (n_jobs <= 0) return cudaSuccess;
    stage_direct<C, Q><<<n_jobs, C::NT, direct_smem<C, Q>(), st>>>(a);
    return cudaGetLastError();
}

template <class C, int Q>
cudaError_t prepare_direct_t() {
    return cudaFuncSetAttribute(stage_direct<C, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)direct_smem<C, Q>());
}

template <class C, int Q>
StageVariant make_direct_variant(const char* name) {
    static_assert(C::NTP == 0 && C::TC == 0, "the direct form runs the plain gather and epilogue");
    StageVariant v = make_variant<C>(name);
    v.smem = (int)direct_smem<C, Q>();
    v.direct = Q;
    v.launch = &launch_direct_t<C, Q>;
    v.prepare = &prepare_direct_t<C, Q>;
    v.smem_for = &direct_smem_for<C, Q>;
    return v;
}

// appended after every other form of the length (indices of the existing
// variants stay as they are)
const StageVariant* stage_variants_direct(int L, int* n) {
    static const StageVariant v128[] = {
        make_direct_variant<Cfg<128, 16, 128, 6, 16, 8>, 8>("L128 cs16 nt128 direct q8"),
        make_direct_variant<Cfg<128, 16, 128, 6, 16, 8>, 4>("L128 cs16 nt128 direct q4"),
        make_direct_variant<Cfg<128, 32, 256, 3, 16, 8>, 8>("L128 cs32 nt256 direct q8"),
        make_direct_variant<Cfg<128, 8, 64, 8, 16, 8>, 8>("L128 cs8 nt64 direct q8"),
    };
    switch (L) {
        case 128: *n = 4; return v128;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
