// misc.cu -- per-step kernels around the stage kernels, and the variant
// registry.
#include <cuda_runtime.h>

#include <vector>

#include "launch.hpp"

namespace pstd {

const StageVariant* stage_variants_small(int L, int* n);
const StageVariant* stage_variants_mid(int L, int* n);
const StageVariant* stage_variants_large(int L, int* n);
const StageVariant* stage_variants_huge(int L, int* n);

const StageVariant* stage_variants_fused_s(int L, int* n);
const StageVariant* stage_variants_fused_m(int L, int* n);
const StageVariant* stage_variants_fused_l(int L, int* n);
const StageVariant* stage_variants_fused_h(int L, int* n);

const StageVariant* stage_variants_direct(int L, int* n);
const StageVariant* stage_variants_toeplitz(int L, int* n);
const StageVariant* stage_variants_toeplitz_ws(int L, int* n);

const StageVariant* stage_variants_tma_a(int L, int* n);
const StageVariant* stage_variants_tma_b(int L, int* n);

static const StageVariant* stage_variants_tma(int L, int* n) {
    if (L <= 512) return stage_variants_tma_a(L, n);
    return stage_variants_tma_b(L, n);
}

static const StageVariant* stage_variants_fused(int L, int* n) {
    if (L <= 256) return stage_variants_fused_s(L, n);
    if (L <= 1024) return stage_variants_fused_m(L, n);
    if (L <= 2048) return stage_variants_fused_l(L, n);
    return stage_variants_fused_h(L, n);
}

// Per length: the fused-form variants first (the default when nothing is
// tuned), then the TMA-staged persistent forms, then the split gather /
// transform / epilogue forms, then the precision-study variants, then the
// direct-convolution forms of short strips (CUDA cores, then tcgen05).  Built once, before any launch.
int stage_variants(int L, const StageVariant** out) {
    static const std::vector<std::vector<StageVariant>> lists = [] {
        std::vector<std::vector<StageVariant>> all(14);
        for (int lg = 0; lg < 14; lg++) {
            const int len = 1 << lg;
            int nf = 0, nt = 0, n = 0;
            const StageVariant* f = stage_variants_fused(len, &nf);
            const StageVariant* tv = stage_variants_tma(len, &nt);
            const StageVariant* v = nullptr;
            if (len <= 256) v = stage_variants_small(len, &n);
            else if (len <= 1024) v = stage_variants_mid(len, &n);
            else if (len <= 2048) v = stage_variants_large(len, &n);
            else v = stage_variants_huge(len, &n);
            for (int i = 0; i < nf; i++) all[lg].push_back(f[i]);
            for (int i = 0; i < nt; i++) all[lg].push_back(tv[i]);
            for (int i = 0; i < n; i++) all[lg].push_back(v[i]);
            int nd = 0;
            const StageVariant* dv = stage_variants_direct(len, &nd);
            for (int i = 0; i < nd; i++) all[lg].push_back(dv[i]);
            const StageVariant* ev = stage_variants_toeplitz(len, &nd);
            for (int i = 0; i < nd; i++) all[lg].push_back(ev[i]);
            const StageVariant* wv = stage_variants_toeplitz_ws(len, &nd);
            for (int i = 0; i < nd; i++) all[lg].push_back(wv[i]);
        }
        return all;
    }();
    *out = nullptr;
    if (L <= 0 || (L & (L - 1)) || L >= (1 << 14)) return 0;
    int lg = 0;
    while ((1 << lg) < L) lg++;
    const auto& v = lists[lg];
    if (v.empty()) return 0;
    *out = v.data();
    return (int)v.size();
}

// After the sixth stage, for every PML domain (kernel/Solver.cpp:85,
// kernel/core/Domain.cpp:716-725): keep p0 = px + py from before the multiply
// (the reference does not recompute p0 after it), then px *= ax, py *= ay.
// vx and vy of non-rigid domains were attenuated in the stage epilogue; rigid
// domains (fields in the fixed buffer) get all four multiplies here.
// one (row, 128-column chunk) block `lb` of PML domain doms[idx[dj]]
__device__ __forceinline__ void pml_post_block(int dj, int lb, const int* idx, const DevDomain* doms, float* set,
                                               float* fixed, float* p0, const float* __restrict__ att) {
    const DevDomain d = doms[idx[dj]];
    float* base = d.fixed ? fixed : set;
    const int chunks = (d.nx + 1 + 127) >> 7;   // vx rows have nx + 1 columns
    const int r = lb / chunks, i = ((lb - r * chunks) << 7) + threadIdx.x;
    if (r < d.ny && i < d.nx) {
        const long long e = (long long)r * d.pitch_p + i;
        const float px = base[d.o_px + e], py = base[d.o_py + e];
        p0[d.o_p0 + e] = __fadd_rn(px, py);
        if (d.att_xp >= 0) base[d.o_px + e] = __fmul_rn(px, att[d.att_xp + i]);
        if (d.att_yp >= 0) base[d.o_py + e] = __fmul_rn(py, att[d.att_yp + r]);
    }
    if (d.fixed) {
        if (r < d.ny && i < d.nx + 1 && d.att_xv >= 0) {
            const long long e = d.o_vx + (long long)r * d.pitch_vx + i;
            base[e] = __fmul_rn(base[e], att[d.att_xv + i]);
        }
        if (r < d.ny + 1 && i < d.nx && d.att_yv >= 0) {
            const long long e = d.o_vy + (long long)r * d.pitch_vy + i;
            base[e] = __fmul_rn(base[e], att[d.att_yv + r]);
        }
    }
}

// the domain of flat block b: the last k with off[k] <= b (off ascends, off[0] = 0)
__device__ __forceinline__ int pml_domain_of(const int* off, int n, int b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void pml_post_kernel(const int* idx, int n, const int* off, const DevDomain* doms, float* set,
                                float* fixed, float* p0, const float* __restrict__ att) {
    // one element per thread, one block per (row, 128-column chunk) of a domain.
    // off (prefix sums of the domains' block counts): a flat grid, the block's
    // domain found by binary search; off == nullptr: domain = blockIdx.y.
    int dj = blockIdx.y, lb = blockIdx.x;
    if (off) {
        dj = pml_domain_of(off, n, (int)blockIdx.x);
        lb = blockIdx.x - off[dj];
    }
    pml_post_block(dj, lb, idx, doms, set, fixed, p0, att);
}

// the flat form with the domain and block counts in device memory: a fixed
// grid strides over the blocks
__global__ void pml_post_dev_kernel(const int* idx, const int* counts, const int* off, const DevDomain* doms,
                                    float* set, float* fixed, float* p0, const float* __restrict__ att,
                                    const int* scene_step, const int* scene_limit) {
    const int n = counts[0], blocks = counts[1];
    for (int b = blockIdx.x; b < blocks; b += gridDim.x) {
        const int dj = pml_domain_of(off, n, b);
        const int sc = doms[idx[dj]].scene;
        if (scene_step[sc] >= scene_limit[sc]) continue;   // the same for the whole block
        pml_post_block(dj, b - off[dj], idx, doms, set, fixed, p0, att);
    }
}

// Gaussian speaker initial condition (kernel/core/Speaker.cpp:21-39) on every
// domain, PML included; speakers are added in order.  Writes the initial p0
// array and px, py of the initial set (rigid domains: of the fixed buffer).
__global__ void speaker_kernel(const DevDomain* doms, const int* dom_x0, const int* dom_y0, const DevSpeaker* spk,
                               int n_spk, float dx, float band_width, float* set, float* fixed, float* p0out) {
    const DevDomain d = doms[blockIdx.y];
    const float x0 = (float)dom_x0[blockIdx.y], y0 = (float)dom_y0[blockIdx.y];
    float* base = d.fixed ? fixed : set;
    const int stride = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.nx * d.ny; k += stride) {
        const int j = k / d.nx, i = k - j * d.nx;   // j: row (y), i: column (x)
        float p0 = 0.f, px = 0.f, py = 0.f;
        for (int s = 0; s < n_spk; s++) {
            const float rx = __fsub_rn(spk[s].x, x0), ry = __fsub_rn(spk[s].y, y0);
            const float ax = __fsub_rn(rx, (float)i), ay = __fsub_rn(ry, (float)j);
            // SQR(a*dx) expands to a*dx*a*dx in the reference
            const float sq = __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(ax, dx), ax), dx),
                                       __fmul_rn(__fmul_rn(__fmul_rn(ay, dx), ay), dx));
            const float p = expf(__fmul_rn(-band_width, sq));
            const float ang = atan2f(ax, ay);
            const float c = cosf(ang), sn = sinf(ang);
            p0 = __fadd_rn(p0, p);
            px = __fadd_rn(px, __fmul_rn(__fmul_rn(c, c), p));
            py = __fadd_rn(py, __fmul_rn(__fmul_rn(sn, sn), p));
        }
        const long long e = (long long)j * d.pitch_p + i;
        p0out[d.o_p0 + e] = p0;
        base[d.o_px + e] = px;
        base[d.o_py + e] = py;
    }
}

// One sample per receiver after the step (kernel/core/Receiver.cpp:80-83):
// p0(rel.x, rel.y) of the (non-PML) container, i.e. row rel.x, column rel.y,
// where p0 = px + py of the last stage.
__global__ void receiver_kernel(const DevReceiver* rec, int n_rec, const DevDomain* doms, const float* __restrict__ set,
                                float* ring, int ring_cap, int* counter) {
    const int step = *counter;
    for (int r = threadIdx.x; r < n_rec; r += blockDim.x) {
        const DevReceiver q = rec[r];
        const DevDomain d = doms[q.dom];
        const long long e = (long long)q.row * d.pitch_p + q.col;
        ring[(long long)(step % ring_cap) * n_rec + r] = __fadd_rn(set[d.o_px + e], set[d.o_py + e]);
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = step + 1;
}

// p0 of a cell after the step, as the next step's first stage reads it:
// the stale p0 array of PML domains, else px + py (kernel/Solver.cpp:85)
__device__ __forceinline__ float p0_after_step(const DevDomain& d, const float* set, const float* fixed,
                                               const float* p0, long long e) {
    if (d.pml) return p0[d.o_p0 + e];
    const float* b = d.fixed ? fixed : set;
    return __fadd_rn(b[d.o_px + e], b[d.o_py + e]);
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Spectral receivers, part 1: one warp per stencil row.  The x shift of the
// row to the receiver's column is a fixed linear map of the windowed strip
// (the bands of the x neighbours blended with the row's ends, as the pressure
// derivative gathers them), so it is a dot product with precomputed weights.
__global__ void si_rows_kernel(const DevSiRow* __restrict__ rows, int n_rows, const float* __restrict__ wt,
                               const DevDomain* doms, const float* __restrict__ set, const float* __restrict__ fixed,
                               const float* __restrict__ p0, float* rowval) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n_rows) return;
    const DevSiRow q = rows[i];
    const DevDomain d = doms[q.dom];
    const float* w = wt + q.w;
    float acc = 0.f;
    if (q.d1 >= 0) {
        const DevDomain a = doms[q.d1];
        const long long e = (long long)q.r1 * a.pitch_p + (a.nx - q.W);
        for (int j = lane; j < q.W; j += 32) acc = fmaf(w[j], p0_after_step(a, set, fixed, p0, e + j), acc);
    }
    {
        const long long e = (long long)q.row * d.pitch_p;
        for (int j = lane; j < d.nx; j += 32) acc = fmaf(w[q.W + j], p0_after_step(d, set, fixed, p0, e + j), acc);
    }
    if (q.d2 >= 0) {
        const DevDomain b = doms[q.d2];
        const long long e = (long long)q.r2 * b.pitch_p;
        for (int j = lane; j < q.W; j += 32)
            acc = fmaf(w[q.W + d.nx + j], p0_after_step(b, set, fixed, p0, e + j), acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) rowval[i] = q.yw * acc;
}

// part 2: one warp per receiver sums its rows in FP64 (a fixed order:
// deterministic), rounded once to the float sample
__global__ void si_receiver_kernel(const int* __restrict__ first, int n_rec, const float* __restrict__ rowval,
                                   float* ring, int ring_cap, int* counter) {
    const int step = *counter;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = threadIdx.x >> 5; r < n_rec; r += nw) {
        double acc = 0.0;
        for (int k = first[r] + lane; k < first[r + 1]; k += 32) acc += (double)rowval[k];
        acc = warp_sum(acc);
        if (lane == 0) ring[(long long)(step % ring_cap) * n_rec + r] = (float)acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = step + 1;
}

__global__ void server_receiver_kernel(const DevSrvReceiver* rec, int n_rec, const DevDomain* doms,
                                       const float* __restrict__ set, float* aux, int* scene_step,
                                       const int* scene_limit, const int* slots, int n_slots, const int* counts) {
    if (counts) {
        n_rec = counts[0];
        n_slots = counts[1];
    }
    for (int r = threadIdx.x; r < n_rec; r += blockDim.x) {
        const DevSrvReceiver q = rec[r];
        const long long step = scene_step[q.slot];
        if (step >= scene_limit[q.slot]) continue;   // the ring holds exactly the scene's steps
        const DevDomain d = doms[q.dom];
        const long long e = (long long)q.row * d.pitch_p + q.col;
        aux[q.ring + step * q.stride + q.index] = __fadd_rn(set[d.o_px + e], set[d.o_py + e]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_slots; i += blockDim.x)
        if (scene_step[slots[i]] < scene_limit[slots[i]]) scene_step[slots[i]] += 1;
}

// p0 = px + py of every `sub`-th row and column (sub = 1: the whole domain)
__global__ void frame_kernel(const int* idx, const long long* dst_off, int n, const DevDomain* doms,
                             const float* __restrict__ set, float* dst, int sub, const float* rec_src, int n_rec,
                             float* rec_dst) {
    if (blockIdx.x == 0 && blockIdx.y == 0)   // the step's receiver row rides along
        for (int i = threadIdx.x; i < n_rec; i += blockDim.x) rec_dst[i] = rec_src[i];
    if ((int)blockIdx.y >= n) return;
    const DevDomain d = doms[idx[blockIdx.y]];
    float* out = dst + dst_off[blockIdx.y];
    const int mx = (d.nx + sub - 1) / sub, my = (d.ny + sub - 1) / sub;
    for (int r = blockIdx.x; r < my; r += gridDim.x)
        for (int i = threadIdx.x; i < mx; i += blockDim.x) {
            const long long e = (long long)r * sub * d.pitch_p + (long long)i * sub;
            out[(long long)r * mx + i] = __fadd_rn(set[d.o_px + e], set[d.o_py + e]);
        }
}

cudaError_t launch_pml_post(const int* idx, int n, int blocks, const DevDomain* doms, float* set, float* fixed,
                            float* p0, const float* att, cudaStream_t st, const int* off) {
    if (n <= 0 || blocks <= 0) return cudaSuccess;
    const dim3 grid = off ? dim3(blocks, 1) : dim3(blocks, n);
    pml_post_kernel<<<grid, 128, 0, st>>>(idx, n, off, doms, set, fixed, p0, att);
    return cudaGetLastError();
}

cudaError_t launch_pml_post_dev(const int* idx, const int* counts, const int* off, const DevDomain* doms, float* set,
                                float* fixed, float* p0, const float* att, const int* scene_step,
                                const int* scene_limit, cudaStream_t st) {
    static int grid = 0;
    if (grid == 0) {
        int dev, sms;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = sms * 16;   // 16 blocks of 128 threads per SM
    }
    pml_post_dev_kernel<<<grid, 128, 0, st>>>(idx, counts, off, doms, set, fixed, p0, att, scene_step, scene_limit);
    return cudaGetLastError();
}

cudaError_t launch_speakers(const DevDomain* doms, const int* x0, const int* y0, int n_dom, const DevSpeaker* spk,
                            int n_spk, float dx, float bw, float* set, float* fixed, float* p0, cudaStream_t st) {
    if (n_dom <= 0) return cudaSuccess;
    speaker_kernel<<<dim3(64, n_dom), 256, 0, st>>>(doms, x0, y0, spk, n_spk, dx, bw, set, fixed, p0);
    return cudaGetLastError();
}

cudaError_t launch_receivers(const DevReceiver* rec, int n_rec, const DevDomain* doms, const float* set, float* ring,
                             int cap, int* counter, cudaStream_t st) {
    receiver_kernel<<<1, 256, 0, st>>>(rec, n_rec, doms, set, ring, cap, counter);
    return cudaGetLastError();
}

cudaError_t launch_spectral_receivers(const DevSiRow* rows, int n_rows, const float* weights, const int* first,
                                      int n_rec, const DevDomain* doms, const float* set, const float* fixed,
                                      const float* p0, float* rowval, float* ring, int cap, int* counter,
                                      cudaStream_t st) {
    if (n_rows > 0) si_rows_kernel<<<(n_rows + 7) / 8, 256, 0, st>>>(rows, n_rows, weights, doms, set, fixed, p0, rowval);
    si_receiver_kernel<<<1, 256, 0, st>>>(first, n_rec, rowval, ring, cap, counter);
    return cudaGetLastError();
}

cudaError_t launch_server_receivers(const DevSrvReceiver* rec, int n_rec, const DevDomain* doms, const float* set,
                                    float* aux, int* scene_step, const int* scene_limit, const int* slots,
                                    int n_slots, cudaStream_t st, const int* counts) {
    if (n_slots <= 0 && !counts) return cudaSuccess;
    server_receiver_kernel<<<1, 256, 0, st>>>(rec, n_rec, doms, set, aux, scene_step, scene_limit, slots, n_slots,
                                              counts);
    return cudaGetLastError();
}

cudaError_t launch_frame(const int* idx, const long long* dst_off, int n, const DevDomain* doms, const float* set,
                         float* dst, cudaStream_t st, int sub, const float* rec_src, int n_rec, float* rec_dst) {
    if (n <= 0 && n_rec <= 0) return cudaSuccess;
    frame_kernel<<<dim3(256, std::max(n, 1)), 256, 0, st>>>(idx, dst_off, n, doms, set, dst, sub, rec_src, n_rec,
                                                           rec_dst);
    return cudaGetLastError();
}

}  // namespace pstd
