/*
 * sph_gb300.h -- C ABI of the GB300 SPH step engine.
 *
 * A drop-in third engine behind the reference's engine interface
 * (Murk42/SPHFluidSimulation, SPHFluidSimulation/include/SPH/Core/
 * SimulationEngine.h:35-76).  Each entry point below names the reference
 * member it replaces.  All functions return sph_status and never abort; all
 * pointers are plain host pointers unless the name says _device.
 *
 * Particle layout on the boundary is the reference's 32-byte DynamicParticle
 * (SPHFluidSimulation/include/SPH/Core/Particles.h:9-17): position, pressure,
 * velocity, hash.  Readback is in the caller's input order.
 *
 * Threading: an engine, batch or server object is used by one host thread at
 * a time (or under the caller's lock).  Different objects are independent.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SPH_API __attribute__((visibility("default")))
#else
#define SPH_API
#endif

typedef enum sph_status {
    SPH_OK = 0,
    SPH_ERR_INVALID_ARGUMENT = 1,   /* null pointer, zero h, bad sizes         */
    SPH_ERR_NOT_INITIALIZED = 2,    /* Update before Initialize (ECPU:422-426) */
    SPH_ERR_CUDA = 3,               /* a CUDA runtime call failed              */
    SPH_ERR_OUT_OF_MEMORY = 4,      /* device allocation failed                */
    SPH_ERR_DEVICE_TIMEOUT = 5,     /* a bounded device wait ran out           */
    SPH_ERR_CAPACITY = 6,           /* exceeds a fixed limit of the object     */
    SPH_ERR_BUDGET = 7,             /* HBM budget of a server exhausted        */
    SPH_ERR_NOT_FOUND = 8           /* unknown scene / job id                  */
} sph_status;

/* The scene-supplied fields of ParticleBehaviourParameters
 * (SPHFluidSimulation/include/SPH/Core/Particles.h:19-37; filled from the
 * scene JSON by SceneBlueprint.cpp:15-33).  selfDensity and the smoothing
 * kernel constant are derived by the engine as SimulationEngineCPU.cpp:406-407
 * does. */
typedef struct sph_params {
    float particle_mass;
    float gas_constant;
    float elasticity;              /* carried, unused by the step (as in the reference) */
    float viscosity;
    float gravity_x, gravity_y, gravity_z;
    float rest_density;
    float max_interaction_distance; /* h: smoothing radius and cell size */
} sph_params;

/* Reference DynamicParticle, 32 bytes (Particles.h:9-17). */
typedef struct sph_dynamic_particle {
    float position[3];
    float pressure;
    float velocity[3];
    uint32_t hash;                 /* bucket key of the position (SF:644-645) */
} sph_dynamic_particle;

/* Reference StaticParticle, 16 bytes (Particles.h:19-23). */
typedef struct sph_static_particle {
    float position[3];
    float pressure;
} sph_static_particle;

typedef struct sph_engine sph_engine;

/* Human-readable name of a status code. */
SPH_API const char* sph_status_string(sph_status status);

/* Last error message recorded on this host thread (empty if none). */
SPH_API const char* sph_last_error(void);

/* Engine constructor: replaces SimulationEngineCPU(threadCount)
 * (SimulationEngineCPU.cpp:351-360).  device = CUDA ordinal. */
SPH_API sph_status sph_engine_create(sph_engine** out, int device);

/* Destructor (SimulationEngineCPU.cpp:361-364).  Frees all device memory. */
SPH_API sph_status sph_engine_destroy(sph_engine* engine);

/* SimulationEngine::Clear (SimulationEngineCPU.cpp:365-395): drops the
 * scene, keeps the device arrays.  The next sph_engine_initialize reuses
 * them when the new scene fits (particles, buckets, statics, triangles) and
 * allocates afresh only when it grows. */
SPH_API sph_status sph_engine_clear(sph_engine* engine);

/* SimulationEngine::Initialize (SimulationEngineCPU.cpp:396-419) with the
 * SceneBlueprint flattened to arrays (SceneBlueprint.h:23-51):
 *   dyn_pos     n x 3 floats, the "dynamic" layer positions
 *   dyn_vel     n x 3 floats or NULL (the reference starts at rest)
 *   static_pos  s x 3 floats, the "static" layer positions (may be NULL if s=0)
 *   triangles   t x 9 floats, boundary mesh triangles (may be NULL if t=0)
 *   reorder_time_interval  the scene's "reorderTimeInterval"
 *               (SimulationEngineCPU.cpp:401; FLT_MAX = never reorder).  The
 *               engine keeps particles sorted by bucket in memory every step;
 *               the interval decides, as in the reference, when a particle's
 *               buffer index is renumbered, and that index orders the members
 *               of a bucket in the neighbour passes
 * Bucket count is 2n (SimulationEngineCPU.cpp:486), static buckets s. */
SPH_API sph_status sph_engine_initialize(sph_engine* engine, const sph_params* params,
                                         const float* dyn_pos, const float* dyn_vel, uint32_t n,
                                         const float* static_pos, uint32_t s,
                                         const float* triangles, uint32_t t,
                                         float reorder_time_interval);

/* SimulationEngine::Update (SimulationEngineCPU.cpp:420-459): advance
 * `steps` steps of dt.  Returns when the device work is complete (the
 * reference's CPU engine queues asynchronously and may drop the call; this
 * engine never drops a call). */
SPH_API sph_status sph_engine_update(sph_engine* engine, float dt, uint32_t steps);

/* Same, but returns once the work is queued on the engine's stream. */
SPH_API sph_status sph_engine_update_async(sph_engine* engine, float dt, uint32_t steps);

/* Waits for queued work; reports SPH_ERR_DEVICE_TIMEOUT if a bounded device
 * wait expired during it. */
SPH_API sph_status sph_engine_synchronize(sph_engine* engine);

/* GetDynamicParticlesBufferManager()->LockRead() readback
 * (OfflineCPUParticleBufferManager.cpp:109-115): the current particles in
 * the caller's input order (out has n entries). */
SPH_API sph_status sph_engine_read_dynamic(sph_engine* engine, sph_dynamic_particle* out);

/* The same particles in the reference's own buffer order: out[k] is the
 * particle at index k of SimulationEngineCPU's current buffer (the initial
 * bucket sort, SimulationEngineCPU.cpp:69-128, then renumbered by every
 * reordering step, SF:332-345), i.e. the bytes LockRead() returns there. */
SPH_API sph_status sph_engine_read_dynamic_buffer(sph_engine* engine, sph_dynamic_particle* out);

/* LockWrite()-style upload: replaces every particle's position, pressure and
 * velocity (input order; the hash is recomputed from the position) and
 * re-sorts.  The pressure stays until the next step's density pass. */
SPH_API sph_status sph_engine_write_dynamic(sph_engine* engine, const sph_dynamic_particle* in);

/* The same upload left queued on the engine's stream, like the OpenCL
 * engine's LockWrite(signalEvent) / Unlock(waitEvents) pair
 * (ParticleBufferManager.h:7-25): it returns once the work is enqueued, and
 * `in` must stay unchanged until the next call that waits for the stream
 * (sph_engine_synchronize, sph_engine_update, a read).  Device errors are
 * reported by that call. */
SPH_API sph_status sph_engine_write_dynamic_async(sph_engine* engine, const sph_dynamic_particle* in);

/* GetStaticParticlesBufferManager()->LockRead(): static particles in bucket
 * order, plus the s+1 bucket-start table (may be NULL). */
SPH_API sph_status sph_engine_read_static(sph_engine* engine, sph_static_particle* out, uint32_t* bucket_starts);

/* The dynamic bucket table after the last step, in the reference's meaning
 * (hashMap, SimulationEngineCPU.cpp:486-487): bucket_starts has 2n+1 entries,
 * bucket b holds slots [bucket_starts[b], bucket_starts[b+1]); slot_ids has n
 * entries, the input index of the particle in each slot (the reference's
 * particleMap followed through its init permutation).  Either may be NULL. */
SPH_API sph_status sph_engine_read_buckets(sph_engine* engine, uint32_t* bucket_starts, uint32_t* slot_ids);

/* GetSimulationTime (SimulationEngineCPU.h:23). */
SPH_API sph_status sph_engine_simulation_time(sph_engine* engine, double* seconds);

/* SystemImplementationName (SimulationEngineCPU.h:19): "CUDA-sm_103a". */
SPH_API const char* sph_engine_implementation_name(void);

/* Particle counts: which = 0 dynamic, 1 static, 2 dynamic buckets, 3 triangles. */
SPH_API sph_status sph_engine_count(sph_engine* engine, int which, uint64_t* value);

/* Arithmetic of the neighbour passes.  exact = 0 (the default): fused
 * multiply-adds and reciprocal multiplies; results agree with the reference
 * to rounding (density to about 3e-7 relative).  exact = 1: the reference's
 * own operations one for one (SPHFunctions.cpp:358-656 with IEEE Vec3
 * operators), in the reference's visiting order, so every step reproduces
 * the bits of SimulationEngineCPU run synchronously; the one exception is a
 * pair of particles at the same position, whose RandomDirection uses the
 * sine of the platform's math library.  The exact form costs some speed. */
SPH_API sph_status sph_engine_set_exact(sph_engine* engine, int exact);

/* Debug output: when on, each step also stores the acceleration
 * F/rho + g of every particle; read it (input order, n x 3) after a step. */
SPH_API sph_status sph_engine_record_acceleration(sph_engine* engine, int on);
SPH_API sph_status sph_engine_read_acceleration(sph_engine* engine, float* out);

/* Per-kernel device time of the last update, milliseconds, in the order
 * density, force, scan, scatter, gather (5 values).  Recorded only while
 * timing is on (it adds events to each step). */
SPH_API sph_status sph_engine_set_timing(sph_engine* engine, int on);
SPH_API sph_status sph_engine_kernel_times(sph_engine* engine, float* ms, int count);

/* Neighbour statistics of the current state, for measurement (one extra
 * launch and a synchronisation; no effect on the simulation).  The per-slot
 * walk of the density pass (launch shape 5) tests every dynamic particle of
 * the 27 neighbour buckets it does not skip (SF:397-495 tests all of them):
 * `candidates` counts those tests and `warp_slots` the lane-slots a warp
 * spends on them, since each bucket costs a warp its largest member count.
 * The group walk (the default) tests each slot against every member of its
 * 27 buckets, 32 candidates per lane-slot round: `group_candidates` counts
 * those tests and `group_lane_slots` the lane-slots spent (32 per round);
 * `group_fallback` counts the slots it leaves to the per-slot walk.
 * `neighbours` counts dynamic pairs within h (each ordered pair once),
 * `static_neighbours` static particles within h of a dynamic one. */
typedef struct sph_neighbour_stats {
    uint64_t particles;
    uint64_t candidates;
    uint64_t warp_slots;
    uint64_t neighbours;
    uint64_t static_neighbours;
    uint64_t group_candidates;
    uint64_t group_lane_slots;
    uint64_t group_fallback;
} sph_neighbour_stats;
SPH_API sph_status sph_engine_neighbour_stats(sph_engine* engine, sph_neighbour_stats* out);

/* A step configuration as the autotuner chose it. */
typedef struct sph_launch_config {
    int mode;                  /* 0 persistent fused step, 1 staged step graph */
    uint32_t persistent_ctas;  /* grid of the persistent step (mode 0), else 0 */
    int density_threads;       /* density pass: threads per CTA ...            */
    int density_min_ctas;      /* ... and resident CTAs per SM it is built for */
    int force_threads;         /* the same for the force pass                  */
    int force_min_ctas;
    float ms_per_step;         /* measured by the autotuner (or its cache)     */
    int from_cache;            /* 1: taken from the autotuner's cache          */
    int density_walk;          /* density pass: 0 group walk, 1 per-slot walk  */
} sph_launch_config;

/* The launch autotuner of sph_batch_autotune for one engine's staged step
 * (launch shapes of the density and force passes; the engine does not use
 * the persistent step).  It replaces any sph_engine_save_state copy, since
 * the trials run on that copy.  out may be NULL. */
SPH_API sph_status sph_engine_autotune(sph_engine* engine, uint32_t trial_steps, sph_launch_config* out);

/* Sets the launch shapes of the engine's density and force passes by index
 * (0 = 128 x 7, the default; 1 = 64 x 14; 2 = 256 x 3; 3 = 128 x 6; 4 =
 * 128 x 8; threads per CTA x resident CTAs per SM), as the autotuner does.
 * Density also has shape 5: 128 x 7 with the per-slot walk in place of the
 * group walk.  Results do not depend on the shapes. */
SPH_API sph_status sph_engine_set_launch_shapes(sph_engine* engine, int density_shape, int force_shape);

/* Device-side checkpoint of the scene (one per engine, kept on the device):
 * save copies the sorted particles, their buffer tags and the bucket table,
 * restore puts them back together with the simulation time and the reorder
 * clock, so the steps that follow repeat the saved run bit for bit.  Used to
 * time and profile several passes over the same steps.  The reference has
 * no counterpart (its buffers are the caller's, ParticleBufferManager.h:7-25).
 * A new scene (sph_engine_initialize / clear) discards the copy. */
SPH_API sph_status sph_engine_save_state(sph_engine* engine);
SPH_API sph_status sph_engine_restore_state(sph_engine* engine);

/* Measurement: the GPU's FP32 issue rate, measured by a fused multiply-add
 * microbenchmark (every SM fully occupied, eight independent FMA chains per
 * thread, CUDA-event timed, at least 50 ms).  warp_fma_per_s = warp FMA
 * instructions issued per second over the GPU; ms = the timed launch.  It
 * is the issue-bound roofline of the neighbour passes.  No counterpart in
 * the reference, which publishes no performance figures. */
SPH_API sph_status sph_probe_fp32_issue(int device, double* warp_fma_per_s, float* ms);

/* The engine's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events with the engine's launches. */
SPH_API sph_status sph_engine_get_stream(sph_engine* engine, void** stream);

/* Failure-detection test hook.  Every device wait of the engine (the scan's
 * look-back, the persistent step's grid barrier) gives up after a bounded
 * number of polls, sets a bit in a device status word and lets the kernel
 * finish; the host then reports SPH_ERR_DEVICE_TIMEOUT and the context stays
 * usable.  This call makes one such wait run out: the scan kernel runs for a
 * tile whose predecessor is never published.  It returns
 * SPH_ERR_DEVICE_TIMEOUT with the status bits (1 = scan wait expired) after
 * about a second. */
SPH_API sph_status sph_debug_expire_wait(int device, uint32_t* status_bits);

/* ---- headless particle rendering ----------------------------------------
 * The reference's particle renderer (ParticleRenderer.cpp:75-82 with
 * Shaders/particle.vert:67-117 and particle.frag:17-22) without a graphics
 * stack: each particle is a camera-facing quad of half-size `size` around its
 * view-space centre, cut to the disc inside it; colour mix(color, red,
 * clamp(1 - exp(-pressure/2000), 0, 1)) with alpha faded out within 4-5
 * units of the eye; depth test LESS, first drawn wins ties, drawn in the
 * reference's order (dynamic particles by buffer index, then statics). */
typedef struct sph_render_view {
    float proj[16];      /* u_projMatrix, column-major (element [col*4 + row]) */
    float view[16];      /* u_viewMatrix */
    float model[16];     /* u_modelMatrix */
    uint32_t width, height;
} sph_render_view;

typedef struct sph_render_layer {
    float size;          /* u_size */
    float color[4];      /* u_color, RGBA in [0, 1] */
} sph_render_layer;

/* Renders scene state into host images: rgba (width*height*4 bytes, RGBA8,
 * row 0 at the bottom as in GL window coordinates) and depth (width*height
 * floats, window depth in [0, 1], 1 where nothing was drawn); either may be
 * NULL.  A NULL layer is not drawn.  The reference's application draws the
 * dynamic layer at size 0.1 and the static one at 0.03
 * (SimulationVisualisationScene.cpp:60-61). */
SPH_API sph_status sph_engine_render(sph_engine* engine, const sph_render_view* view,
                                     const sph_render_layer* dynamic_layer, const sph_render_layer* static_layer,
                                     uint8_t* rgba, float* depth);

/* ---- the counting sort stage on its own ---------------------------------
 * Hash + count + scan + scatter of n positions into `buckets` buckets with
 * cell size h, on the device (SF:321-356 with the serial scan of
 * SimulationEngineCPU.cpp:245-253).  Outputs (each may be NULL):
 *   keys    n     key of each input position, GetHash(GetCell(p)) % buckets
 *   counts  buckets  particles per bucket
 *   starts  buckets+1  bucket start slots, starts[buckets] = n
 *   order   n     input index of the particle in each slot; inside a bucket
 *                 by decreasing input index, the slots the reference's fill
 *                 gives (SF:346-356: slot = --count[key] over i = 0..n-1) */
SPH_API sph_status sph_cell_sort(int device, const float* pos, uint32_t n, float h, uint32_t buckets,
                                 uint32_t* keys, uint32_t* counts, uint32_t* starts, uint32_t* order);

/* The same counting sort for callers that cannot allocate device memory
 * (code under a caller-owned pool or allocator, a frame loop that must not
 * allocate, a plugin whose host application owns all device memory).  It has
 * no counterpart in the reference.  Every pointer is a DEVICE pointer owned
 * by the caller: pos n x 3 floats, keys n, starts buckets+1 (16-byte
 * aligned), order n; the outputs mean what sph_cell_sort's do.  Work is
 * queued on `stream` (a cudaStream_t, NULL = default stream) and the call
 * returns after it finished, so it cannot be captured into a CUDA graph: on
 * a capturing stream it queues nothing and returns SPH_ERR_INVALID_ARGUMENT.
 * The sort's scratch is a fixed array inside the library (about 4.2 MiB,
 * held on every GPU that loads the library until the process exits), so the
 * call makes no allocation; n is limited to 262144 and buckets to 524288,
 * larger requests fail with SPH_ERR_CAPACITY.  The first call on a device
 * looks up that array's device address (with the device current); after a
 * cudaDeviceReset the next call looks it up again, since the array then
 * lives in a new context.  All calls share the array: calls that overlap on
 * the GPU race and must be serialised by the caller.  On any status other
 * than SPH_OK the contents of keys, starts and order are undefined. */
SPH_API sph_status sph_cell_sort_noalloc(const float* pos, uint32_t n, float h, uint32_t buckets,
                                         uint32_t* keys, uint32_t* starts, uint32_t* order, void* stream);

/* ---- batched engine: many scenes advanced by one persistent launch ------ */

typedef struct sph_batch sph_batch;

/* Creates an empty batch on `device`. */
SPH_API sph_status sph_batch_create(sph_batch** out, int device);
SPH_API sph_status sph_batch_destroy(sph_batch* batch);

/* Adds a scene (same arguments as sph_engine_initialize plus its dt);
 * returns its id.  Scenes are uploaded when the batch is finalized. */
SPH_API sph_status sph_batch_add_scene(sph_batch* batch, const sph_params* params,
                                       const float* dyn_pos, const float* dyn_vel, uint32_t n,
                                       const float* static_pos, uint32_t s,
                                       const float* triangles, uint32_t t, float dt,
                                       uint32_t* scene_id);

/* Uploads and sorts all scenes, sizes the persistent launch, captures the
 * step in a CUDA graph. */
SPH_API sph_status sph_batch_finalize(sph_batch* batch);

/* Advances every scene by `steps` steps (each by its own dt), one persistent
 * launch per step.  mode 0 = persistent fused step (default), mode 1 = one
 * launch per stage over all scenes. */
SPH_API sph_status sph_batch_step(sph_batch* batch, uint32_t steps);
SPH_API sph_status sph_batch_set_mode(sph_batch* batch, int mode);

/* Neighbour-pass arithmetic of every scene, as sph_engine_set_exact: with
 * exact = 1 each scene's bytes equal the reference CPU engine's. */
SPH_API sph_status sph_batch_set_exact(sph_batch* batch, int exact);

/* The launch autotuner.  It times trial_steps steps of each configuration on
 * a saved copy of the state (restored after each trial, so the simulation
 * does not advance) and keeps the fastest: the staged step graph with the
 * density pass under each launch shape (threads per CTA x register-bound
 * resident CTAs per SM: 128 x 7, the default, 64 x 14, 256 x 3, 128 x 6,
 * 128 x 8), then the force pass under each shape with the best density
 * shape, then the persistent kernel at 1, 2, ... CTAs per SM up to its
 * occupancy limit.  Every shape computes the same bits.  The choice is
 * cached per GPU and size class (log2 of the particle and scene counts,
 * arithmetic) in the process, and in the file named by the environment
 * variable SPH_AUTOTUNE_CACHE when set; a cached class is not timed again.
 * Reports the chosen mode (0 persistent, 1 staged), the persistent grid
 * size (0 when staged) and its time per step (any output may be NULL).
 * The reference sizes its OpenCL launches from device queries instead
 * (SimulationEngineGPUKernels.cpp:260-291). */
SPH_API sph_status sph_batch_autotune(sph_batch* batch, uint32_t trial_steps, int* mode, uint32_t* grid_ctas,
                                      float* ms_per_step);

/* The batch's current configuration (after sph_batch_autotune: its choice). */
SPH_API sph_status sph_batch_launch_config(sph_batch* batch, sph_launch_config* out);

/* Reads one scene's particles in its input order. */
SPH_API sph_status sph_batch_read_scene(sph_batch* batch, uint32_t scene_id, sph_dynamic_particle* out);

/* Sum of particles over scenes; the persistent grid size chosen. */
SPH_API sph_status sph_batch_info(sph_batch* batch, uint64_t* total_particles, uint32_t* grid_ctas,
                                  uint32_t* threads_per_cta);

/* ---- server: continuous batching of simulation jobs -------------------- */

typedef struct sph_server sph_server;

/* hbm_budget_bytes bounds the resident state of admitted jobs; max_slots
 * bounds how many jobs share one step. */
SPH_API sph_status sph_server_create(sph_server** out, int device, uint64_t hbm_budget_bytes,
                                     uint32_t max_slots);
SPH_API sph_status sph_server_destroy(sph_server* server);

/* Queues a job (copied): a scene plus a horizon in steps.  Rejects with
 * SPH_ERR_BUDGET if the job alone can never fit the budget and
 * SPH_ERR_INVALID_ARGUMENT for malformed jobs. */
SPH_API sph_status sph_server_submit(sph_server* server, const sph_params* params,
                                     const float* dyn_pos, uint32_t n,
                                     const float* static_pos, uint32_t s, float dt,
                                     uint32_t steps, uint64_t* job_id);

/* Runs one scheduling round, pipelined with the GPU: waits for the steps
 * the previous round queued and retires the jobs they finished (their
 * readback is queued), admits queued jobs that fit, and queues the next
 * steps -- every admitted job advanced by up to `chunk_steps` steps in one
 * batched launch sequence -- then returns while the GPU runs them.  Keep
 * polling until *active and *queued are 0: the round that finishes the last
 * jobs is retired by the poll after it.  *active and *queued report the
 * state afterwards. */
SPH_API sph_status sph_server_poll(sph_server* server, uint32_t chunk_steps, uint32_t* active,
                                   uint32_t* queued);

/* Neighbour-pass arithmetic of every job, as sph_engine_set_exact. */
SPH_API sph_status sph_server_set_exact(sph_server* server, int exact);

/* Ids of the jobs retired since the last call, oldest first: up to
 * `capacity` of them are moved into job_ids and *count says how many (the
 * rest stay for the next call).  A caller polls, then fetches just these. */
SPH_API sph_status sph_server_finished(sph_server* server, uint64_t* job_ids, uint32_t capacity,
                                       uint32_t* count);

/* Retrieves a finished job's particles (input order, n entries) and
 * densities (n floats, rho = p/k + rho0); may be NULL.  Returns
 * SPH_ERR_NOT_FOUND while the job is unfinished. */
SPH_API sph_status sph_server_result(sph_server* server, uint64_t job_id, sph_dynamic_particle* out,
                                     float* density);

/* Bytes of device state a job of n dynamic and s static particles holds. */
SPH_API uint64_t sph_server_job_bytes(uint32_t n, uint32_t s);

/* Where the polls' host time went, for measurement: phase_seconds[6] =
 * admission (uploads and sort launches), waiting for the admissions' sorts,
 * rebuilding the scene table and step graph, queueing the steps, waiting for
 * the steps (their device time), reading finished jobs back; counts[3] =
 * polls, steps run, scene-table rebuilds.  Either may be NULL. */
SPH_API sph_status sph_server_stats(sph_server* server, double* phase_seconds, uint64_t* counts);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
