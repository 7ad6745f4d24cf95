// launch.hpp -- host-side view of the kernels: stage-kernel variants and the
// small per-step kernels.
#pragma once
#include <cuda_runtime.h>

#include "device.cuh"

namespace pstd {

struct StageArgs {
    const DevJob* jobs;
    const DevDomain* doms;
    const float* in;        // state after the previous stage (derivative input)
    const float* prev;      // stage-start state
    float* out;             // new state
    const float* fixed;     // fields of rigid domains
    const float* p0;        // per-domain p0 read at the first stage (initial / stale)
    const int* first_step;  // per scene: 1 while the scene's very first step runs
    const float2* filt;     // derivative filters (position order); jobs index them by dtab
    const float2* filt_p;   // this bucket's pressure and velocity filters (persistent form)
    const float2* filt_v;
    const float* win;       // window coefficients
    const float2* tw;       // twiddles exp(-2 pi i j / L), j < L
    const float* att;       // PML attenuation profiles
    int stage;              // 0..5
    int last;               // 1 at the sixth stage
    int row_cap;            // pipelined / staged forms: floats staged per strip (>= strip length + 2, multiple of 4)
    // staged (TMA) form: 2-D tensor maps of every domain's fields (PSTD_TMAP_BYTES
    // each, index (domain * 4 + field) * 4 + set, p0 as field 0 of set 3), the
    // state-set indices of `in` and `prev`, and the word a CTA sets when a staged
    // copy does not complete in time
    const unsigned char* maps;
    int set_in, set_prev;
    int* err;
    // serving loop, persistent form: per-scene steps taken and step limits; a
    // job of a scene that has taken all its steps is skipped (null: none skip)
    const int* scene_step = nullptr;
    const int* scene_limit = nullptr;
};

constexpr int PSTD_TMAP_BYTES = 128;   // sizeof(CUtensorMap)

#if defined(__CUDACC__)
#define PSTD_HD __host__ __device__
#else
#define PSTD_HD
#endif
// staged form: floats staged per strip for a bucket row cap rc (whole 16-byte
// quads of a row job's strips, whole boxes of a column job's strips), and the
// rows of one tensor-map box of a field with `rows` rows
PSTD_HD constexpr int tma_cap(int rc) { return rc <= 256 ? (rc + 7) / 8 * 8 : (rc + 255) / 256 * 256; }
PSTD_HD constexpr int tma_box_rows(int rows) { return rows < 256 ? (rows + 7) / 8 * 8 : 256; }

// One compiled shape of the stage kernel for one transform length.
struct StageVariant {
    int L, CS, NT, smem, np;
    int r[4];                                                   // radix of each pass
    bool persistent;                                            // warp-specialised persistent form
    bool pipe;                                                  // pipelined persistent form (cp.async staging)
    bool bf16;                                                  // split-BF16 tensor-core DFT (precision study, opt-in)
    int shf = 0;                                                // fused form: last radix split over a lane pair (shuffles)
    bool tma = false;                                           // staged form: needs tensor maps and a row cap
    int ctw = 0;                                                // twiddle tables hold powers (Cfg::CTW)
    bool tc5 = false;                                           // tcgen05 TF32x3 DFT (precision study, opt-in)
    int direct = 0;                                             // direct convolution, Q outputs per task (filter: h)
    cudaError_t (*launch)(int n_jobs, const StageArgs& a, cudaStream_t st);
    cudaError_t (*prepare)();
    size_t (*smem_for)(int row_cap);                            // dynamic shared memory of one CTA
    const char* name;
    // persistent form over a job table whose length is read from device
    // memory at launch time (serving loop; null where not compiled): resident
    // CTAs take jobs from *counter, skip all-zero jobs and jobs of scenes at
    // their step limit
    cudaError_t (*launch_dev)(const int* count, const StageArgs& a, int* counter, cudaStream_t st) = nullptr;
    cudaError_t (*prepare_dev)() = nullptr;
};

// all variants compiled for length L (nullptr / 0 if L is not supported)
int stage_variants(int L, const StageVariant** out);

// merged form (stage_all.cu): one persistent launch per RK stage over the jobs
// of every length 128..2048; CTAs take jobs from *counter (zeroed before the
// stage); jobs carry their own length and twiddle-table offset
bool merged_supports(int L);
// configuration family fam: 0 = 256 threads, 3 CTAs per SM; 1 = 128 threads,
// 8 CTAs per SM, computed twiddles (PSTD_MERGED_FAMILY picks the default)
int merged_family_default();
const StageVariant* merged_variant(int L, int fam);
cudaError_t prepare_stage_all(int fam);
cudaError_t launch_stage_all(int fam, int n_jobs, const StageArgs& a, int* counter, cudaStream_t st);
// the same over two job tables in one array, counts read from device memory
// at launch time: counts[0] jobs at a.jobs[0..), then counts[1] jobs at
// a.jobs[counts[2]..) (all resident CTAs start; zero counts are an empty
// stage).  All-zero jobs (length 0, no copy flag) are skipped.
cudaError_t launch_stage_all_dev(int fam, const int* counts, const StageArgs& a, int* counter, cudaStream_t st);

// serving loop, per-length persistent form (stage_serve.cu): one compiled
// configuration per transform length 32..8192 with launch_dev set (nullptr
// for other lengths)
const StageVariant* serve_variant(int L);

// one block per (row, 128-column chunk): with off (n + 1 prefix sums of the
// domains' (rows + 1) x ceil((columns + 1) / 128) block counts) blocks is their
// total; without, blocks is the count of the largest domain (grid blocks x n)
cudaError_t launch_pml_post(const int* doms_idx, int n, int blocks, const DevDomain* doms, float* set, float* fixed,
                            float* p0, const float* att, cudaStream_t st, const int* off = nullptr);
// the same with n and blocks read from device memory (counts[0], counts[1]) by a
// fixed grid that strides over the blocks; domains of scenes that have taken
// all their steps (scene_step >= scene_limit) are left alone
cudaError_t launch_pml_post_dev(const int* doms_idx, const int* counts, const int* off, const DevDomain* doms,
                                float* set, float* fixed, float* p0, const float* att, const int* scene_step,
                                const int* scene_limit, cudaStream_t st);
cudaError_t launch_speakers(const DevDomain* doms, const int* x0, const int* y0, int n_dom, const DevSpeaker* spk,
                            int n_spk, float dx, float bw, float* set, float* fixed, float* p0, cudaStream_t st);
cudaError_t launch_receivers(const DevReceiver* rec, int n_rec, const DevDomain* doms, const float* set, float* ring,
                             int cap, int* counter, cudaStream_t st);
// spectral receivers: every stencil row's x-shifted, y-weighted p0 into rowval
// (one warp per row), then receiver r's sample = the sum of rowval over
// rows [first[r], first[r + 1]) into the ring, and the counter + 1
cudaError_t launch_spectral_receivers(const DevSiRow* rows, int n_rows, const float* weights, const int* first,
                                      int n_rec, const DevDomain* doms, const float* set, const float* fixed,
                                      const float* p0, float* rowval, float* ring, int cap, int* counter,
                                      cudaStream_t st);
// serving loop: one sample per receiver into its scene's ring at the scene's
// step count, then every listed slot's step count + 1 -- only for scenes below
// their step limit (counts: n_rec and n_slots read from device memory,
// counts[0] and counts[1])
cudaError_t launch_server_receivers(const DevSrvReceiver* rec, int n_rec, const DevDomain* doms, const float* set,
                                    float* aux, int* scene_step, const int* scene_limit, const int* slots, int n_slots,
                                    cudaStream_t st, const int* counts = nullptr);
// dense p0 = px + py of the given domains into dst (frames); sub > 1 keeps
// every sub-th row and column (ceil(nx/sub) x ceil(ny/sub) values per domain);
// n_rec floats of rec_src (a receiver row) are copied to rec_dst on the way
cudaError_t launch_frame(const int* doms_idx, const long long* dst_off, int n, const DevDomain* doms, const float* set,
                         float* dst, cudaStream_t st, int sub = 1, const float* rec_src = nullptr, int n_rec = 0,
                         float* rec_dst = nullptr);

}  // namespace pstd
