/*
 * pstd_gb300.h -- C ABI of the GB300-native PSTD solve.
 *
 * This is the drop-in boundary for openPSTD's kernel API.  Every entry point
 * replaces one piece of the reference's C++ interface (paths are relative to
 * the openPSTD source tree):
 *
 *   pstd_create          <- PSTDKernel::initialize_kernel   (kernel/PSTDKernel.cpp:49-59)
 *   pstd_run             <- PSTDKernel::run + GPUSingleThreadSolver::compute_propagation
 *                           (kernel/PSTDKernel.cpp:121-148, kernel/Solver.cpp:62-93,153-156)
 *   pstd_get_metadata    <- PSTDKernel::get_metadata        (kernel/PSTDKernel.cpp:154-168)
 *   pstd_destroy         <- ~PSTDKernel
 *   pstd_callbacks       <- KernelCallback / KernelCallbackLog (kernel/KernelInterface.h:243-304)
 *   pstd_config          <- PSTDConfiguration / PSTDSettings / DomainConf
 *                           (kernel/KernelInterface.h:44-240)
 *
 * Extra entry points (device-resident stepping, snapshots, scene inspection,
 * batched multi-scene solves and the serving loop) have no single reference
 * counterpart; each says so.
 *
 * Conventions: every function returns an int status (PSTD_OK == 0); no C++
 * exception crosses this boundary.  pstd_last_error() gives a message for the
 * last failing call on the calling thread.  All pointers are host pointers
 * unless a parameter name says "dev".  Grid axes follow the reference: x is
 * the column index, y the row index, fields are stored row-major (x fastest)
 * when they cross this boundary.
 */
#ifndef PSTD_GB300_H
#define PSTD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PSTD_OK                 0
#define PSTD_ERR_INVALID        1  /* bad argument or malformed configuration */
#define PSTD_ERR_NOT_CONFIGURED 2  /* PSTDKernelNotConfiguredException (kernel/PSTDKernel.cpp:122-123) */
#define PSTD_ERR_CUDA           3  /* a CUDA runtime call failed */
#define PSTD_ERR_UNSUPPORTED    4  /* scene makes the reference read undefined memory (see message) */
#define PSTD_ERR_CALLBACK       5  /* a callback returned non-zero: run stopped between frames */
#define PSTD_ERR_NO_MEMORY      6  /* device or pinned host allocation failed / over budget */
#define PSTD_ERR_CANCELLED      7  /* request cancelled */
#define PSTD_ERR_TIMEOUT        8  /* a bounded device wait gave up */
#define PSTD_ERR_IO             9  /* the scene file's key/value store failed (see pstd_file_last_error) */

/* ---- log levels (KernelCallbackLog, kernel/KernelInterface.h:243-271) --- */
#define PSTD_LOG_FATAL   0
#define PSTD_LOG_ERROR   1
#define PSTD_LOG_WARNING 2
#define PSTD_LOG_INFO    3
#define PSTD_LOG_DEBUG   4

/* ---- configuration (PSTDSettings, kernel/KernelInterface.h:44-158) ----- */
typedef struct pstd_settings {
    float calctime;        /* render time [s]                         */
    float c1;              /* sound speed [m/s]                       */
    float ampMax;          /* PML attenuation coefficient             */
    float freqMax;         /* maximum frequency (not used by the solve) */
    float rho;             /* density of air [kg/m^3]                 */
    float patcherror;      /* patch error [dB]; sets window size      */
    float tfactRK;         /* CFL factor; dt = tfactRK*dx/c1          */
    float gridSpacing;     /* dx = dy [m]                             */
    float band_width;      /* Gaussian speaker band width [1/m^2]     */
    float wave_length;     /* (only used by spectral interpolation)   */
    float rk_coefficients[6];
    int32_t n_rk_coefficients;     /* must be 6 */
    int32_t spectral_interpolation;/* 0 / 1: nearest-neighbour receivers, as the reference, which reads its
                                      flag but hard-disables the interpolation (kernel/core/Receiver.cpp:48);
                                      PSTD_RECEIVERS_SPECTRAL: spectral interpolation (see below) */
    int32_t PMLCells;
    int32_t SaveNth;
} pstd_settings;

/* Spectral receivers (no reference counterpart that runs: the reference's
 * Receiver::compute_with_si, kernel/core/Receiver.cpp:85-121, is disabled and
 * shifts by the integer grid location, :41).  The receiver at grid location
 * (gx, gy) = world / dx, in the cell (ix, iy) = ((int)gx, (int)gy) of its
 * container, samples p0 at the point itself: p0 of the container and of its
 * low and high y neighbours is shifted along x by gx - ix with the windowed
 * strip transform of the pressure derivative (Domain::calc's bands,
 * reflection / transmission and window, factors exp(i k (gx - ix) dx) in
 * place of the derivative's), and the shifted column ix is shifted along y by
 * gy - iy the same way.  Not available in the serving loop and in
 * pstd_solve_noalloc. */
#define PSTD_RECEIVERS_SPECTRAL 2

/* DomainConfEdge (kernel/KernelInterface.h:163-175) */
typedef struct pstd_domain_edge {
    float absorption;
    int32_t lr;            /* locally reacting flag */
} pstd_domain_edge;

/* DomainConf (kernel/KernelInterface.h:180-205); world units [m] */
typedef struct pstd_domain_conf {
    float top_left[2];
    float size[2];
    pstd_domain_edge T, L, B, R;
} pstd_domain_conf;

/* PSTDConfiguration (kernel/KernelInterface.h:213-240) */
typedef struct pstd_config {
    pstd_settings settings;
    int32_t n_domains;
    const pstd_domain_conf* domains;
    int32_t n_speakers;
    const float* speakers;   /* 3*n_speakers floats, world (x, y, z) */
    int32_t n_receivers;
    const float* receivers;  /* 3*n_receivers floats, world (x, y, z) */
} pstd_config;

/* ---- callbacks (KernelCallback, kernel/KernelInterface.h:279-304) ------- */
/* write_frame: data is row-major (x fastest), n = Nx*Ny floats of p0 of a
 *   non-PML domain, valid only for the duration of the call (copy to keep).
 *   Called when frame % SaveNth == 0, before PML attenuation (kernel/Solver.cpp:80-84).
 * write_sample: n == 1 sample of receiver `receiver` at time step start_sample
 *   (kernel/Solver.cpp:86-91).
 * frame_buffer (optional, no reference counterpart): asked for a frame's
 *   destination when the frame is formed, some frames before its write_frame;
 *   returns host memory for n floats that stays untouched by the caller until
 *   write_frame(frame, domain) hands the same pointer back, filled (the
 *   caller then owns it: no copy).  Memory pinned or registered with
 *   pstd_host_register is copied into directly by the device; NULL (or a
 *   NULL callback) uses the library's own staging and write_frame's data is
 *   valid only during the call.
 * A non-zero return stops the run at the next frame boundary with
 * PSTD_ERR_CALLBACK.  log and frame_buffer may be NULL. */
typedef struct pstd_callbacks {
    void* user;
    int (*write_frame)(void* user, int32_t frame, int32_t domain, const float* data, int64_t n);
    int (*write_sample)(void* user, int32_t start_sample, int32_t receiver, const float* data, int64_t n);
    void (*log)(void* user, int32_t level, const char* message);
    float* (*frame_buffer)(void* user, int32_t frame, int32_t domain, int64_t n);
} pstd_callbacks;

/* Page-lock host memory for direct device copies (frame_buffer destinations);
 * wraps cudaHostRegister / cudaHostUnregister.  No reference counterpart. */
int pstd_host_register(void* ptr, int64_t bytes);
int pstd_host_unregister(void* ptr);

typedef struct pstd_kernel pstd_kernel;

/* Build the scene (domains, automatic PML, speakers, receivers, attenuation
 * tables) on the host and upload it to device 0.  The stage-kernel plan is
 * autotuned (PSTD_AUTOTUNE=0 disables it) at the first create of a scene
 * structure in the process and taken from a per-process plan cache afterwards.
 * Replaces PSTDKernel::initialize_kernel (kernel/PSTDKernel.cpp:49-70). */
int pstd_create(const pstd_config* config, const pstd_callbacks* log_cb, pstd_kernel** out);

/* Replaces PSTDKernel::~PSTDKernel. Safe on NULL. */
void pstd_destroy(pstd_kernel* k);

/* Replaces PSTDKernel::get_metadata (kernel/PSTDKernel.cpp:154-168).
 * dims receives 3 ints (x, y, z=0) per scene domain, PML included, in scene
 * order; at most `cap` domains are written, *n_domains gets the total. */
int pstd_get_metadata(pstd_kernel* k, int32_t* n_domains, int32_t* dims, int32_t cap, int32_t* framecount);

/* Replaces PSTDKernel::run with the GPU solver (kernel/PSTDKernel.cpp:121-148,
 * kernel/Solver.cpp:62-93).  Runs Framecount time steps from the current
 * state, emitting frames and receiver samples through cb.  Blocks the
 * calling thread; callbacks run on it, in frame order.  The device runs
 * ahead of the callbacks by as many frames as fit in 64 MiB (at least 3, at
 * most 8): each is copied to pinned host memory on a copy stream while later
 * steps compute. */
int pstd_run(pstd_kernel* k, const pstd_callbacks* cb);

/* pstd_run with frame subsampling on the device (no reference counterpart):
 * frames every save_nth-th step (0 = the scene's SaveNth, kernel/Solver.cpp:80)
 * and, for stride > 1, only every stride-th row and column of each domain, so
 * write_frame gets ceil(Nx/stride) * ceil(Ny/stride) floats, row-major.
 * Cuts the device-to-host traffic of runs that do not need every frame at
 * full resolution; receiver samples are unchanged. */
int pstd_run_sub(pstd_kernel* k, const pstd_callbacks* cb, int32_t save_nth, int32_t stride);

/* ---- device-resident stepping (no reference counterpart) --------------- */
/* Advance n_steps time steps on `stream` (a cudaStream_t, NULL = the handle's
 * own stream) without callbacks.  Receiver samples are kept on the device
 * (readable with pstd_get_receivers).  Asynchronous: returns after enqueue. */
int pstd_advance(pstd_kernel* k, int32_t n_steps, void* stream);

/* Re-initialise the fields to the state right after pstd_create (speaker
 * initial condition, zero velocities, step counter 0). Asynchronous on the
 * handle's stream. */
int pstd_reset(pstd_kernel* k);

/* Synchronise the handle's stream. */
int pstd_synchronize(pstd_kernel* k);

/* Number of time steps taken so far. */
int pstd_steps_done(pstd_kernel* k, int32_t* steps);

/* Copy receiver samples [first_step, first_step+n_steps) x n_receivers into
 * dst (step-major).  Only steps taken since the last pstd_reset that are
 * still in the device ring (capacity set at create: Framecount) are valid. */
int pstd_get_receivers(pstd_kernel* k, int32_t first_step, int32_t n_steps, float* dst);

/* Field codes for pstd_snapshot */
#define PSTD_FIELD_P0 0
#define PSTD_FIELD_PX 1
#define PSTD_FIELD_PY 2
#define PSTD_FIELD_VX 3   /* Ny x (Nx+1) */
#define PSTD_FIELD_VY 4   /* (Ny+1) x Nx */

/* Copy one field of scene domain `domain_index` (scene order, PML included)
 * to dst, row-major, dense.  n must equal the field's element count. */
int pstd_snapshot(pstd_kernel* k, int32_t domain_index, int32_t field, float* dst, int64_t n);

/* ---- batched solves (no reference counterpart) --------------------------
 * Several independent scenes advanced together: every RK stage launches
 * the stage kernel once per strip length over the strips of all scenes.
 * Domains and receivers of the batch are numbered globally, scene after
 * scene; pstd_advance / pstd_get_receivers / pstd_snapshot / scene
 * inspection take these global indices.  pstd_run is single-scene only. */
int pstd_create_batch(const pstd_config* configs, int32_t n_configs, const pstd_callbacks* log_cb, pstd_kernel** out);
/* info[5] = {first global domain, domains, first global receiver, receivers, Framecount} */
int pstd_batch_scene(pstd_kernel* k, int32_t scene, int32_t* info);
int pstd_batch_size(pstd_kernel* k, int32_t* n_scenes, int32_t* n_receivers);

/* ---- scene inspection (no reference counterpart; used for parity tests) - */
typedef struct pstd_domain_info {
    int32_t id;
    int32_t top_left[2];
    int32_t size[2];
    int32_t is_pml, is_secondary_pml, is_rigid, local;
    int32_t should_update[2];       /* [X, Y] */
    int32_t n_neighbours[4];        /* LEFT, RIGHT, TOP, BOTTOM (kernel/core/kernel_functions.h:94-96) */
    int32_t fft_length[2];          /* X, Y strip transform length (0 if not updated) */
    int32_t window[2];              /* window length after halving, X, Y */
    float alpha, impedance, rho;
} pstd_domain_info;

/* Build only the host-side scene (no device state, no GPU needed) so that
 * the scene can be inspected; device calls on such a handle return
 * PSTD_ERR_NOT_CONFIGURED.  Release with pstd_destroy. */
int pstd_scene_build(const pstd_config* config, pstd_kernel** out);
/* Strip plan of a domain: number of interface runs along axis (0 x, 1 y) and
 * for each run (first strip, count, low neighbour, high neighbour); -1 = none. */
int pstd_scene_strip_runs(pstd_kernel* k, int32_t index, int32_t axis, int32_t* runs, int32_t cap, int32_t* n);
int pstd_scene_domain_count(pstd_kernel* k, int32_t* n);
int pstd_scene_domain_info(pstd_kernel* k, int32_t index, pstd_domain_info* out);
/* dir: 0 LEFT 1 RIGHT 2 TOP 3 BOTTOM; writes scene indices of the neighbours */
int pstd_scene_neighbours(pstd_kernel* k, int32_t index, int32_t dir, int32_t* out, int32_t cap, int32_t* n);
/* PML attenuation vectors of a domain: ax_p[Nx], ax_v[Nx+1], ay_p[Ny], ay_v[Ny+1]
 * (1 where the domain is not attenuated along that axis). */
int pstd_scene_attenuation(pstd_kernel* k, int32_t index, float* ax_p, float* ax_v, float* ay_p, float* ay_v);

/* ---- timing of the stage kernels (no reference counterpart) ------------ */
/* Advance n_steps with CUDA events around every RK stage (its strip-length
 * launches concurrent, as in the step graphs); returns the summed device time
 * [ms] of the stages, the time of the whole region, and the launch counts.
 * Results are identical to pstd_advance. */
int pstd_profile_passes(pstd_kernel* k, int32_t n_steps, void* stream,
                        float* ms_stage, float* ms_total, int32_t* stage_launches, int32_t* total_launches);

/* Stage-kernel plan: one line per strip-length bucket (length, jobs,
 * variant chosen by the autotuner with its index, the timings it compared). */
int pstd_plan_info(pstd_kernel* k, char* buf, int32_t cap);

/* The stage-kernel variants compiled for transform length L, one line per
 * variant: "<index> <name>" (the index PSTD_PLAN=L:index pins).  Host only:
 * no GPU needed.  *n (may be NULL) = number of variants. */
int pstd_stage_variants(int32_t L, char* buf, int32_t cap, int32_t* n);

/* The round-trip gain per frequency bin (natural order, k < L) of the stage
 * kernel's transform with passes radices[0..np) (last pass in registers),
 * computed twiddles (ctw) or the last radix split over a lane pair
 * (lane_pair), from the rounding of its float constants; the derivative
 * filters are divided by it.  out: 2 L doubles (re, im).  Host only. */
int pstd_transform_gain(int32_t L, const int32_t* radices, int32_t np, int32_t ctw, int32_t lane_pair, double* out);

/* Counts that define the work: cells advanced per step (pressure cells of
 * non-rigid domains), of which air cells, and the number of kernel launches
 * per time step. */
int pstd_work_counts(pstd_kernel* k, int64_t* cells, int64_t* air_cells, int32_t* launches_per_step);

/* ---- serving loop (no counterpart in the reference) ----------------------
 * Continuous batching of scene solves on one GPU.  The server reserves
 * hbm_budget_bytes of device memory once (three state-set arenas, p0, rigid
 * fields, receiver rings) and keeps at most max_scenes scenes active.
 * pstd_server_submit builds the scene on the host and queues it; every
 * pstd_server_tick admits queued requests in arrival order while their
 * fields fit (admission by HBM footprint), advances all active scenes
 * together and hands finished scenes' receiver series (and, with
 * PSTD_REQ_FINAL_FRAME, their last p0 frame) to the host.  By default every
 * RK stage is one persistent stage-kernel launch per strip length over
 * device-resident job tables that admissions and completions update in
 * place (the step graphs are captured again only when a table grows or a
 * new strip length appears); a tick runs up to max_steps steps and each
 * scene stops on the device at its own step count.  PSTD_SERVE_FORM=merged
 * uses one merged launch per stage; PSTD_SERVE_PERSISTENT=0 rebuilds the
 * plan per membership change and advances all scenes to the nearest
 * completion.  Results equal a solo pstd_create + pstd_advance of the same
 * scene with the same kernel configurations.  One thread drives a server;
 * calls are not re-entrant. */
typedef struct pstd_server pstd_server;
#define PSTD_REQ_QUEUED    0
#define PSTD_REQ_ACTIVE    1
#define PSTD_REQ_DONE      2
#define PSTD_REQ_CANCELLED 3
#define PSTD_REQ_FINAL_FRAME 1   /* submit flag: keep p0 of the non-PML domains after the last step */
int pstd_server_create(int64_t hbm_budget_bytes, int32_t max_scenes, const pstd_callbacks* log_cb, pstd_server** out);
void pstd_server_destroy(pstd_server* s);
/* PSTD_ERR_NO_MEMORY if the scene alone exceeds the arenas */
int pstd_server_submit(pstd_server* s, const pstd_config* config, int32_t n_steps, int32_t flags, int64_t* request_id);
/* info (may be NULL): {active, queued, finished in this tick, steps advanced} */
int pstd_server_tick(pstd_server* s, int32_t max_steps, int32_t* info);
/* sizes (may be NULL): {receiver floats = n_steps x n_receivers, frame floats} */
int pstd_server_poll(pstd_server* s, int64_t request_id, int32_t* state, int32_t* steps_done, int64_t* sizes);
/* copy a finished request's results (sizes as pstd_server_poll reports) and forget it */
int pstd_server_result(pstd_server* s, int64_t request_id, float* receivers, int64_t n_receivers, float* frame,
                       int64_t n_frame);
int pstd_server_cancel(pstd_server* s, int64_t request_id);
/* stats[8] = {budget bytes, bytes in use, peak bytes in use, cell-steps done,
 *             requests done, plan rebuilds, active, queued} */
int pstd_server_stats(pstd_server* s, int64_t* stats);
/* launch form: out[4] = {CUDA graph captures, in-place table updates (membership
 * changes served without a capture), 1 if the current step is the persistent
 * form (one merged launch per RK stage, counts read from device memory),
 * kernel launches per step} */
int pstd_server_launch_stats(pstd_server* s, int64_t* out);

/* ---- allocation-free solve (no counterpart in the reference) ------------
 * For callers that cannot allocate device memory: host applications that
 * own the GPU's memory through their own pool or arena (a serving process
 * whose caching allocator has reserved the HBM, an engine with a fixed
 * device-memory budget) and real-time loops, for which cudaMalloc / cudaFree
 * may fail under the host's budget and synchronise the device.
 *
 * Builds `config` on the host, advances n_steps (>= 1) time steps from the
 * speaker initial condition on `stream` (a cudaStream_t, NULL = the legacy
 * default stream) and writes, when the pointers are not NULL:
 *   frame_dev      p0 after the last step of every non-PML domain, in scene
 *                  order, each Nx*Ny row-major -- the values pstd_run hands
 *                  write_frame for that frame (frame_len >= their total);
 *   receivers_dev  n_steps x n_receivers samples, step-major, as
 *                  pstd_get_receivers returns them (receivers_len >= that).
 * Both are DEVICE pointers owned by the caller; results are ready when the
 * stream's work completes.  The call allocates no device memory: state
 * sets, tables and plan live in one static device array of
 * PSTD_NOALLOC_SCRATCH_BYTES per device, held from module load until the
 * process exits.  Scenes that need more are rejected with PSTD_ERR_INVALID
 * and a message giving the bytes needed (use pstd_create for those).
 * The first call on a device takes the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the
 * process.  A cudaDeviceReset unloads the array with the module, so that
 * address no longer holds: after a reset, do not call this entry point
 * again in the same process.  Every call shares the array and clears it
 * itself; calls whose GPU work overlaps (other streams, other threads on one
 * device) race on it.  The plan upload is a pageable host-to-device copy,
 * so the call waits for work already queued on `stream`.  Each strip length
 * runs the first one-CTA-per-job FP32 stage-kernel variant compiled for it
 * (no autotuning; pstd_create with PSTD_VARIANT=0 runs the same ones), so
 * results match pstd_create + pstd_advance to FP32 rounding. */
#define PSTD_NOALLOC_SCRATCH_BYTES (16u << 20)
int pstd_solve_noalloc(const pstd_config* config, int32_t n_steps, float* frame_dev, int64_t frame_len,
                       float* receivers_dev, int64_t receivers_len, void* stream);

/* The stencils of a scene's spectral receivers, built on the host (no device
 * needed; no reference counterpart).  Receiver r's sample after a step is
 *   sum over rows i in [first[r], first[r+1]) of
 *     row_weights[i] * (  sum_j<W  weights[w + j]          p0[d1](r1, nx(d1) - W + j)
 *                       + sum_j<nx weights[w + W + j]      p0[dom](row, j)
 *                       + sum_j<W  weights[w + W + nx + j] p0[d2](r2, j) )
 * with rows[8 i ..] = {dom, row, d1, d2, r1, r2, W, w} (domain indices as
 * pstd_get_metadata lists them, -1 = no band), nx = nx(dom), p0(row, column)
 * the domain's p0 as the next step's first stage reads it.  With all arrays
 * NULL, sizes[0..2] receive the row, weight and receiver counts; otherwise
 * sizes holds the capacities (rows: 8 x sizes[0] int32, row_weights:
 * sizes[0], weights: sizes[1], first: sizes[2] + 1). */
int pstd_spectral_plan(const pstd_config* config, int32_t* rows, float* row_weights, float* weights, int32_t* first,
                       int64_t* sizes);

/* ---- scene files (.pstd) -------------------------------------------------
 * The reference's PSTDFile (shared/PSTDFile.h:161-415, shared/PSTDFile.cpp):
 * an unqlite key/value file holding the scene configuration (a Boost text
 * archive of PSTDConfiguration), per-domain result frames and per-receiver
 * samples under int32 keys {prefix, indices...}.  unqlite is loaded at run
 * time from `unqlite_lib` (NULL: $PSTD_UNQLITE_LIB, else "libunqlite.so"),
 * the shared library the reference builds from its unqlite/unqlite.c.
 * Errors: PSTD_ERR_INVALID (bad argument, missing record, malformed archive),
 * PSTD_ERR_UNSUPPORTED (library missing, wrong file version -- the
 * reference's PSTDFileVersionException), PSTD_ERR_IO (store failure --
 * PSTDFileIOException); pstd_file_last_error() has the message. */
typedef struct pstd_file pstd_file;
/* PSTDFile::Open (create_new = 0; the file must hold version 4) or
 * PSTDFile::New (create_new = 1: version, CreateDefaultConf scene, empty
 * results scene, committed) -- shared/PSTDFile.cpp:168-205 */
int pstd_file_open(const char* path, const char* unqlite_lib, int32_t create_new, pstd_file** out);
void pstd_file_close(pstd_file* f);   /* unqlite_close commits pending changes */
/* GetSceneConf / GetResultsSceneConf (results = 1); the arrays `out` points
 * into stay valid until the next call of this function or pstd_file_close */
int pstd_file_get_scene(pstd_file* f, int32_t results, pstd_config* out);
/* SetSceneConf (results = 0) or the results-scene record (results = 1) */
int pstd_file_set_scene(pstd_file* f, int32_t results, const pstd_config* config);
int pstd_file_initialize_results(pstd_file* f);   /* InitializeResults (:234-249) */
int pstd_file_delete_results(pstd_file* f);       /* DeleteResults (:251-266) */
/* SaveNextResultsFrame: appends frame (count)++ of `domain` (:227-232) */
int pstd_file_save_frame(pstd_file* f, int32_t domain, const float* data, int64_t n);
int pstd_file_frame_count(pstd_file* f, int32_t domain, int32_t* count);   /* GetResultsFrameCount */
/* GetResultsFrame: *n = floats in the record; at most cap copied to dst (dst may be NULL) */
int pstd_file_get_frame(pstd_file* f, int32_t domain, int32_t frame, float* dst, int64_t cap, int64_t* n);
int pstd_file_append_samples(pstd_file* f, int32_t receiver, const float* data, int64_t n);   /* SaveReceiverData */
int pstd_file_get_samples(pstd_file* f, int32_t receiver, float* dst, int64_t cap, int64_t* n);   /* GetReceiverData */
int pstd_file_commit(pstd_file* f);     /* Commit */
int pstd_file_rollback(pstd_file* f);   /* Rollback */
const char* pstd_file_last_error(void);
/* The Boost text archive of `config` alone (no reference counterpart: the
 * reference writes it inside SetSceneConf); *len = its length, at most
 * cap - 1 bytes and a terminating 0 written to buf (buf may be NULL). */
int pstd_archive_encode(const pstd_config* config, char* buf, int64_t cap, int64_t* len);

/* ---- library ------------------------------------------------------------ */
const char* pstd_last_error(void);
const char* pstd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PSTD_GB300_H */
