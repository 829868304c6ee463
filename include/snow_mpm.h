/*
 * snow_mpm.h -- C ABI of the GB300-native explicit snow-MPM step.
 *
 * The library replaces the explicit time-integration stage of MeyerFabian/snow:
 *
 *   reference                                          this ABI
 *   ---------------------------------------------------------------------------
 *   TimeUpdate(PhysicalScene&&) + init() + update(dt)   snow_scene_create / _upload /
 *     (src/snow/simulation/timeUpdate.hpp:10-18)          snow_scene_init / snow_scene_step
 *   ExplicitTimeUpdate::init                            snow_scene_init
 *     (src/snow/simulation/timeUpdate/explicittimeupdate.cpp:4-34)
 *   ExplicitTimeUpdate::update(double dt)               snow_scene_step(scene, dt, 1)
 *     (explicittimeupdate.cpp:36-63)
 *   SemiImplicitTimeUpdate (empty in the reference:     snow_params.implicit_beta > 0
 *     semiimplicittimeupdate.cpp:3-5)                      (FAST mode; snow_scene_solver_report)
 *   Technique::dispatch_with_barrier per kernel         snow_dispatch(scene, SNOW_K_*, dt)
 *     (src/snow/simulation/computingTechnique/*.cpp)
 *   ParticleSystem::initSSBO std140 buffers             snow_scene_upload_std140 /
 *     (src/snow/object/particlesystem.cpp:101-228)        snow_scene_download_std140
 *   CollisionObjects::initSSBO cx/cv/cn                 snow_collider (48 bytes = cx, cv, cn)
 *     (src/snow/object/collisionObjects.cpp:25-66)
 *   defines.hpp constants                               snow_params_default
 *     (src/snow/utils/defines.hpp:14-54)
 *   launchSnow's six wall half-planes                   snow_default_walls
 *     (src/snow/utils/launchHelper/explicit.cpp:9-67)
 *
 * Conventions: the caller owns every host array; the library owns device
 * memory and runs on one CUDA stream per context. Calls return snow_status
 * (0 = success, negative = error; snow_last_error gives the text). No C++
 * exception crosses the ABI. A context is used by one host thread at a time.
 * Matrices in the plain (non-std140) calls are N x 9 row-major floats:
 * F[p][r][c] at 9p + 3r + c.
 */
#ifndef SNOW_MPM_H
#define SNOW_MPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum snow_status {
  SNOW_OK = 0,
  SNOW_EINVAL = -1,       /* invalid argument */
  SNOW_ENOMEM = -2,       /* device allocation failed */
  SNOW_EBUDGET = -3,      /* the context's HBM budget would be exceeded */
  SNOW_ETIMEDOUT = -4,    /* a bounded wait expired */
  SNOW_ENUMERIC = -5,     /* NaN / Inf particle state detected */
  SNOW_ECUDA = -6,        /* CUDA runtime error */
  SNOW_ESTATE = -7,       /* call out of order (step before init, ...) */
  SNOW_EUNSUPPORTED = -8, /* not available in this scene's mode */
  SNOW_ECAPACITY = -9     /* sparse grid block pool overflowed */
} snow_status;

typedef enum snow_mode {
  /* The shaders' arithmetic: int32 fixed-point grid and particle
   * accumulators (x1e8 / x1e6, truncating), V rounded to 1e-5 in the SVD,
   * R / F_E / F_P rounded to 1e-9, dense grid, std140 device buffers. */
  SNOW_MODE_REFERENCE = 0,
  /* FP32 throughout with float accumulation, no quantisation, J_p tracked as
   * a scalar, sparse blocked grid, shared-memory tiled P2G. */
  SNOW_MODE_FAST = 1
} snow_mode;

/* Kernels of one explicit step, named after the reference's Techniques. */
typedef enum snow_kernel {
  SNOW_K_RIGID_ADVANCE = 0, /* rigidAdvance.glsl      */
  SNOW_K_G_RESET = 1,       /* gReset.glsl            */
  SNOW_K_P2G = 2,           /* p2gTransfer.glsl       */
  SNOW_K_G_FORCE = 3,       /* gForceCompute.glsl     */
  SNOW_K_G2P = 4,           /* g2pTransfer.glsl       */
  SNOW_K_P_ADVANCE = 5,     /* particleAdvance.glsl   */
  SNOW_K_G_MASS = 6,        /* gMassCompute.glsl      */
  SNOW_K_P_VOLUME = 7       /* pVolumeCompute.glsl    */
} snow_kernel;

typedef struct snow_params {
  float grid_pos[3];      /* GRID_POS_X/Y/Z                       */
  int grid_dim[3];        /* GRID_DIM_X/Y/Z                       */
  float grid_spacing;     /* GRID_SPACING                         */
  float young;            /* YOUNG_MODULUS  (E0)                  */
  float poisson;          /* POISSON        (nu)                  */
  float hardening;        /* HARDENING      (xi)                  */
  float crit_compression; /* CRIT_COMPRESSION (theta_c)           */
  float crit_stretch;     /* CRIT_STRETCH     (theta_s)           */
  float alpha;            /* PIC/FLIP blend, 0.95 in the shaders  */
  float gravity[3];       /* (0, -9.81, 0) in gForceCompute.glsl  */
  int mode;               /* snow_mode                            */
  int sort_interval;      /* FAST: re-bin particles at least every k steps (0 = library
                           * default). snow_scene_step re-bins every step while particles
                           * leave their work items' tiles between binnings (fast particles,
                           * long steps) and returns to k once they stay put */
  /* Semi-implicit velocity update (the reference's SemiImplicitTimeUpdate,
   * an empty stub in semiimplicittimeupdate.cpp:3-5; Stomakhin et al. 2013,
   * eq. 9): with implicit_beta > 0 each step solves
   * (M + beta dt^2 K) v = M v* on the grid by conjugate residuals before
   * G2P. 0 keeps the explicit step. FAST mode only. */
  float implicit_beta;      /* 0 (explicit) .. 1 (backward Euler)             */
  float implicit_tolerance; /* stop at |r| <= tol |M^1/2 v*| (0 = 1e-5)      */
  int implicit_max_iters;   /* at most this many iterations a step (0 = 50, <= 128) */
} snow_params;

/* One collision object: the reference's cx = (pos, type), cv = (vel,
 * radius), cn = (normal, friction) vec4 triple. type 0 = half-plane through
 * pos with normal; type 1 = sphere of radius about pos. */
typedef struct snow_collider {
  float pos[3];
  int32_t type;
  float vel[3];
  float radius;
  float normal[3];
  float friction;
} snow_collider;

/* Bulk statistics of one scene (for horizons where trajectories diverge). */
typedef struct snow_stats {
  double mass;              /* sum m_p                  */
  double momentum[3];       /* sum m_p v_p              */
  double kinetic_energy;    /* sum 0.5 m_p |v_p|^2      */
  double center_of_mass[3];
  double bbox_min[3], bbox_max[3];
  double mean_jp;           /* mean det F_P             */
  uint64_t nonfinite;       /* particles with a NaN / Inf field */
  uint64_t n;
} snow_stats;

/* Device-timed phases of snow_scene_step when profiling is on (ms, summed
 * over steps since the last reset). `binnings` counts the steps that
 * re-binned the particles (profiling on or off); `wide` the particles whose
 * P2G contributions outgrew the fixed-point scales' fast range and were
 * scattered with int64 contributions (FAST; reading it waits for the
 * stream). */
typedef struct snow_phase_times {
  double sort_ms, p2g_ms, grid_ms, g2p_ms, other_ms, total_ms;
  uint64_t steps;
  uint64_t binnings;
  uint64_t wide;
} snow_phase_times;

typedef struct snow_ctx snow_ctx;
typedef struct snow_scene snow_scene;
typedef struct snow_batch snow_batch;

/* defines.hpp defaults; mode = SNOW_MODE_FAST. */
void snow_params_default(snow_params* p);
/* The six wall half-planes of explicit.cpp:9-67 for p's grid; returns 6. */
int snow_default_walls(const snow_params* p, snow_collider out[6]);

snow_status snow_ctx_create(int device, size_t hbm_budget_bytes, snow_ctx** out);
/* Also destroys every scene and batch of the context still alive; their
 * handles are invalid afterwards. */
void snow_ctx_destroy(snow_ctx* ctx);
const char* snow_last_error(const snow_ctx* ctx);
size_t snow_ctx_bytes_in_use(const snow_ctx* ctx);
snow_status snow_ctx_set_profiling(snow_ctx* ctx, int on);
/* on = 0: snow_scene_step launches each step's kernels one by one instead of
 * replaying the step's captured CUDA graph (default on). Batches always
 * replay graphs. */
snow_status snow_ctx_set_graphs(snow_ctx* ctx, int on);
/* The cudaStream_t every call of this context launches on, for callers that
 * order or time their own GPU work against it. */
void* snow_ctx_stream(const snow_ctx* ctx);
snow_status snow_ctx_synchronize(snow_ctx* ctx);

/* A scene holds up to `capacity` particles (0 = take n from the first upload). */
snow_status snow_scene_create(snow_ctx* ctx, const snow_params* p, const snow_collider* colliders,
                              int n_colliders, size_t capacity, snow_scene** out);
/* Also destroys the batches that hold this scene. */
void snow_scene_destroy(snow_scene* s);
/* Device bytes a scene with these parameters and n particles will hold at
 * most (in SNOW_MODE_FAST the output pool counted at its largest). */
size_t snow_scene_footprint(const snow_params* p, size_t n);

/* x, v: N x 3; m: N; FE, FP: N x 9 row-major or NULL for identity; N >= 1
 * (SNOW_EINVAL otherwise). FAST mode reads arrays in page-locked (pinned)
 * host memory in place; pageable ones are copied to a device staging buffer
 * first. The arrays may be reused once the call returns. */
snow_status snow_scene_upload(snow_scene* s, const float* x, const float* v, const float* m, const float* FE,
                              const float* FP, size_t n);
/* The reference's buffers as ParticleSystem::initSSBO fills them: pxm N x
 * vec4 (x, m), pv N x ivec4 (v*1e8, density*1e6), pFE / pFP N x mat4
 * (column-major). */
snow_status snow_scene_upload_std140(snow_scene* s, const float* pxm, const int32_t* pv, const float* pFE,
                                     const float* pFP, size_t n);
/* Sets the initial particle volume V0 = m / rho0 (N floats) instead of
 * letting snow_scene_init derive it from the first grid mass (pVolumeCompute).
 * Call after an upload and before snow_scene_init; init then keeps it. Used to
 * resume a scene from a saved state. */
snow_status snow_scene_set_volume(snow_scene* s, const float* volume, size_t n);
/* ExplicitTimeUpdate::init: grid reset, grid mass, particle density. */
snow_status snow_scene_init(snow_scene* s);
/* n_steps x ExplicitTimeUpdate::update(dt). Asynchronous: returns once the
 * work is queued. Conditions counted on the device (non-finite particles:
 * SNOW_ENUMERIC, grid block pool overflow: SNOW_ECAPACITY, an expired
 * bounded wait: SNOW_ETIMEDOUT) are returned by a later step call, at the
 * second re-binning point after they occurred (the counters are read there
 * without waiting for the queued steps); snow_scene_stats counts non-finite
 * particles at once. CUDA errors surface at the next call that synchronises
 * (download, stats, snow_ctx_synchronize). */
snow_status snow_scene_step(snow_scene* s, double dt, int n_steps);
/* Waits for the scene's queued work and returns the first condition its
 * device counters hold (SNOW_ETIMEDOUT, SNOW_ECAPACITY, SNOW_ENUMERIC) or
 * SNOW_OK: the same checks snow_scene_step makes at its re-binning points,
 * at once. (No counterpart in the reference, which reports no errors.) */
snow_status snow_scene_check(snow_scene* s);
/* Bounded waits of the FAST kernels. A work item's wait for the bulk copies
 * of its grid tile into shared memory gives up after `wait_ns` nanoseconds
 * of the GPU's global timer (0 = the default, one second): the CTA stops
 * without reading the tile, waits once more (bounded) for copies still in
 * flight, and returns; the scene's next check returns SNOW_ETIMEDOUT and its
 * state is no longer a valid step (the context stays usable). `unsent_bytes`
 * is 0 in normal use: a positive value makes every such wait expect that
 * many bytes more than its copies deliver, so that the wait runs out, to
 * test this path (at most 65536). FAST mode only. (No counterpart in the
 * reference.) */
snow_status snow_scene_set_wait_limit(snow_scene* s, uint32_t wait_ns, uint32_t unsent_bytes);
/* One kernel of the step (per-kernel parity checks). In SNOW_MODE_FAST the
 * gather and the particle update are one kernel: SNOW_K_G2P runs both and
 * SNOW_K_P_ADVANCE does nothing; SNOW_K_G_RESET does nothing (the block pool
 * is cleared as the grid update consumes it). */
snow_status snow_dispatch(snow_scene* s, int kernel, double dt);

/* Any pointer may be NULL. FP is only kept in SNOW_MODE_REFERENCE (FAST
 * returns SNOW_EUNSUPPORTED if FP is requested); Jp = det F_P; volume =
 * initial particle volume m / rho0. */
snow_status snow_scene_download(snow_scene* s, float* x, float* v, float* FE, float* FP, float* Jp, float* volume);
snow_status snow_scene_download_std140(snow_scene* s, float* pxm, int32_t* pv, float* pFE, float* pFP);
/* Dense G = X*Y*Z grid arrays after P2G / the grid update: mass G, momentum
 * G x 3, force G x 3, vstar G x 3 (post-collision velocity). */
snow_status snow_scene_download_grid(snow_scene* s, float* mass, float* momentum, float* force, float* vstar);
snow_status snow_scene_download_colliders(snow_scene* s, snow_collider* out);
snow_status snow_scene_stats(snow_scene* s, snow_stats* out);
/* The same statistics without waiting: snow_scene_stats_enqueue queues them
 * into one of the context's SNOW_STATS_SLOTS slots (after the work already
 * queued on the context's stream) and returns; snow_ctx_stats_read waits for
 * that slot and returns them. A stepping loop can read step i's statistics
 * while step i + 1 runs. Enqueueing into a slot that holds unread statistics
 * waits for them first. (No counterpart in the reference.) */
#define SNOW_STATS_SLOTS 8
snow_status snow_scene_stats_enqueue(snow_scene* s, int slot);
snow_status snow_ctx_stats_read(snow_ctx* ctx, int slot, snow_stats* out);
size_t snow_scene_size(const snow_scene* s);

/* Particle -> cell binning as used by the FAST path: per-particle block-major
 * cell key (block (i>>2, j>>2, k>>2) numbered x fastest, times 64, plus
 * (i&3) + 4(j&3) + 16(k&3), cell = trunc((x - grid_pos)/h) clamped to the
 * grid) and the stable sort permutation (perm[k] = particle at rank k).
 * Computed on the device from the current positions. */
snow_status snow_scene_cell_keys(snow_scene* s, uint32_t* keys, uint32_t* perm);

snow_status snow_scene_phase_times(snow_scene* s, snow_phase_times* out, int reset);

/* The semi-implicit solve of the last step: iterations taken and the
 * relative residuals |r|/|M^1/2 v*| of the mass-scaled system before and
 * after (waits for the stream; SNOW_EUNSUPPORTED for an explicit scene).
 * A step whose solve starts below 1e-3 of its tolerance (it exits at once:
 * v = v*) makes the next steps take v = v* without evaluating the
 * stiffness: 15 steps, doubled for each further factor of 10 below, up to
 * 240. Those steps report 0 iterations and residuals 0, and the step after
 * them checks again. */
typedef struct snow_solver_report {
  int iterations;
  int max_iters;
  double residual;
  double initial_residual;
} snow_solver_report;
snow_status snow_scene_solver_report(snow_scene* s, snow_solver_report* out);

/* ---- Serving ---------------------------------------------------------------
 * A worker thread that owns one context and runs simulation jobs: it admits
 * queued jobs in arrival order while their device footprint fits the HBM
 * budget, keeps every admitted job's state resident, and advances all
 * admitted jobs together as one batch (snow_batch_step) in chunks of steps;
 * jobs that arrive meanwhile join at the next chunk boundary and finished jobs
 * leave, freeing their memory. With a particle cap, only the first resident
 * jobs (arrival order, or least remaining work) step in a chunk; the others
 * keep their state on the device and wait. (No counterpart in the reference,
 * which runs one scene per process.) */
typedef struct snow_server snow_server;

enum { SNOW_SERVE_FIFO = 0, SNOW_SERVE_SRPT = 1 };

typedef struct snow_server_config {
  int device;
  size_t hbm_budget_bytes;      /* admission limit for resident jobs (0 = no limit) */
  int max_active;               /* most jobs resident at once (0 = 256) */
  int chunk_steps;              /* steps per batch launch between admissions (0 = 16) */
  size_t max_active_particles;  /* particles stepped together per chunk (0 = all resident jobs) */
  int policy;                   /* which resident jobs step first under the cap: SNOW_SERVE_* */
} snow_server_config;

typedef struct snow_job_desc {
  const snow_params* params;  /* mode is forced to SNOW_MODE_FAST */
  const snow_collider* colliders;
  int n_colliders;
  const float* x; /* N x 3 */
  const float* v; /* N x 3 */
  const float* m; /* N */
  size_t n;
  int steps;
  double dt;
  int keep_state; /* keep the final state for snow_server_fetch */
} snow_job_desc;

typedef struct snow_job_result {
  uint64_t id;
  int status;          /* snow_status of the job */
  size_t n;
  int steps;
  double queue_s;      /* arrival -> admission */
  double service_s;    /* admission -> completion */
  double latency_s;    /* arrival -> completion */
  snow_stats stats;    /* bulk statistics of the final state */
} snow_job_result;

typedef struct snow_server_report {
  uint64_t submitted, admitted, completed, failed;
  uint64_t pending, active;
  double particle_steps;  /* completed particle-steps of all jobs */
  double busy_s;          /* time with at least one admitted job */
  double uptime_s;
  size_t resident_bytes;
} snow_server_report;

snow_status snow_server_create(const snow_server_config* cfg, snow_server** out);
/* Stops the worker after the jobs already admitted finish; pending jobs are
 * dropped. */
void snow_server_destroy(snow_server* srv);
/* Copies the job's host arrays; returns at once with the job id. */
snow_status snow_server_submit(snow_server* srv, const snow_job_desc* job, uint64_t* id);
/* Moves up to max finished jobs into out; *n_out = how many. */
snow_status snow_server_poll(snow_server* srv, snow_job_result* out, int max, int* n_out);
/* Final state of a finished job submitted with keep_state (x, v: N x 3, FE:
 * N x 9 row-major, Jp: N; any may be NULL); releases it. */
snow_status snow_server_fetch(snow_server* srv, uint64_t id, float* x, float* v, float* FE, float* Jp);
snow_status snow_server_stats(snow_server* srv, snow_server_report* out);
/* Blocks until no job is pending or active, or timeout_s passes
 * (SNOW_ETIMEDOUT). */
snow_status snow_server_drain(snow_server* srv, double timeout_s);

/* Largest key count snow_sort_keys_static accepts. */
#define SNOW_SORT_STATIC_MAX_KEYS 262144

/* The binning sort without any device allocation. (No counterpart in the
 * reference, which has no sort.)
 *
 * For callers that cannot allocate device memory: an application that owns
 * every device buffer up front (for example particle buffers it shares with
 * its renderer) and does not let a plug-in call cudaMalloc, which can
 * synchronise the device and stall a real-time frame loop, or code running
 * under an external memory budget. Everything else in this library allocates
 * through its context; this call needs no context.
 *
 * Sorts n 32-bit keys (device memory, `key_bits` significant low bits,
 * 1..32) stably: sorted_keys receives the keys in ascending order and perm[i]
 * the input index of the i-th smallest key (ties keep input order, as
 * std::stable_sort). `keys` may be the same array as `sorted_keys` (sorted
 * in place); any other overlap between the three arrays, including `perm`
 * sharing memory with either key array, returns SNOW_EINVAL and queues
 * nothing. The work is queued on `stream` (a cudaStream_t; NULL = the
 * default stream) and the call returns without waiting.
 *
 * Scratch lives in one fixed device array inside the library, sized for
 * SNOW_SORT_STATIC_MAX_KEYS keys (about 2.1 MB, held by every GPU that loads
 * the library until the process exits). n above that limit returns
 * SNOW_EINVAL and queues nothing. All calls share the array, so calls whose
 * work overlaps on the GPU (other streams, other host threads) race and must
 * be ordered by the caller; every pass overwrites the scratch it reads, so
 * nothing carried over from an earlier call needs clearing. The first call in
 * a device context (and the first after that device's context was reset)
 * looks up the array's device address; make that first call before any
 * stream capture. Returns SNOW_ECUDA if a CUDA call fails. */
snow_status snow_sort_keys_static(const uint32_t* keys, uint32_t* sorted_keys, uint32_t* perm, size_t n,
                                  int key_bits, void* stream);

/* Batched stepping of many independent scenes (all SNOW_MODE_FAST): one
 * launch per phase covers every scene, the whole step is a CUDA graph. */
snow_status snow_batch_create(snow_ctx* ctx, snow_scene* const* scenes, int n, snow_batch** out);
void snow_batch_destroy(snow_batch* b);
/* dt: one per scene (NULL = each scene's last dt or 1e-3). */
snow_status snow_batch_step(snow_batch* b, const double* dt, int n_steps);
/* Work decomposition of the FAST step (no counterpart in the reference). */
typedef struct snow_tuning {
  int sort_interval;   /* steps between re-binnings of each scene's particles (1..64) */
  int items_max;       /* most particles per work item (64..256) */
  int ctas_per_sm;     /* work-item CTAs per SM (1 or 2) */
  int steps_taken;     /* autotune: steps the batch advanced while timing */
  double ms_per_step;  /* autotune: measured time per step of the choice */
} snow_tuning;
/* Applies a tuning to one FAST scene; the scene's next step re-bins its
 * particles with it (and so starts a new re-binning interval). */
snow_status snow_scene_set_tuning(snow_scene* s, const snow_tuning* t);
/* Applies a tuning to every scene of the batch (e.g. one kept from an
 * earlier autotune); the batch's next step starts the re-binning cycle
 * again (scene i re-bins at cycle step i mod sort_interval). */
snow_status snow_batch_set_tuning(snow_batch* b, const snow_tuning* t);
/* Times candidate tunings (sort interval 1/2/4/8/12/16/24/32 x 128/256 particles per work
 * item x 1/2 CTAs per SM) on real steps of the batch and keeps the fastest;
 * each candidate is timed in a forward and in a reversed pass over the list
 * (the scenes evolve meanwhile, and the two passes cancel a linear drift).
 * The steps advance the scenes like snow_batch_step (out->steps_taken says
 * how many); dt as for snow_batch_step. */
snow_status snow_batch_autotune(snow_batch* b, const double* dt, snow_tuning* out);

#ifdef __cplusplus
}
#endif

#endif /* SNOW_MPM_H */
