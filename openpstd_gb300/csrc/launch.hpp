// launch.hpp -- host launchers of the kernels in kernels.cu.
#pragma once
#include <cuda_runtime.h>

#include "device.cuh"

namespace pstd {

struct PassArgs {
    const DevJob* jobs;
    const DevDomain* doms;
    const float* in;      // state of the previous stage (derivative input)
    const float* prev;    // stage-start state
    float* out;           // new state
    const float2* filt;   // derivative filters (position order)
    const float* win;     // window coefficients
    const float2* tw;     // twiddles exp(-2 pi i j / L), j < L
    const float* att;     // PML attenuation profiles
    int stage;            // 0..5
    int last;             // 1 at the sixth stage
};

// strips per CTA for transform length L (0 if L is not supported)
int pass_strips_per_job(int L);
// radix sequence of the in-place transform of length L
void pass_radices(int L, int* r, int* np);
// allow the pass kernels their dynamic shared memory (call before capture)
cudaError_t prepare_pass_kernels();
cudaError_t launch_pass(int L, int n_jobs, const PassArgs& a, cudaStream_t st);
cudaError_t launch_copy(const DevCopy* copies, int n, const DevDomain* doms, const float* prev, float* out,
                        const float* att, int last, cudaStream_t st);
cudaError_t launch_speakers(const DevDomain* doms, const int* x0, const int* y0, int n_dom, const DevSpeaker* spk,
                            int n_spk, float dx, float bw, float* set, cudaStream_t st);
cudaError_t launch_receivers(const DevReceiver* rec, int n_rec, const DevDomain* doms, const float* set, float* ring,
                             int cap, int* counter, cudaStream_t st);

}  // namespace pstd
