// sph_api.cu -- the C ABI (include/sph_gb300.h) for the single-scene engine,
// the counting-sort stage and the batch.
//
// The engine mirrors SPH::SimulationEngine (reference SPHFluidSimulation/
// include/SPH/Core/SimulationEngine.h:35-76) as implemented by
// SimulationEngineCPU (SimulationEngineCPU.cpp:351-504): Initialize uploads
// and bucket-sorts the scene, Update advances it, readback returns the
// reference's 32-byte particles.
#include <cstring>
#include <memory>
#include <new>

#include "sph_state.h"

using sph::SceneInput;
using sph::StepMode;
using sph::StepState;

struct sph_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    StepState state;
    bool initialized = false;
    double sim_time = 0.0;
    float reorder_interval = 0.f;   // "reorderTimeInterval" (SimulationEngineCPU.cpp:401)
    float reorder_elapsed = 0.f;    // reorderParticlesElapsedTime
    bool record_accel = false;
    bool timing = false;
    bool accel_valid = false;
    uint32_t n = 0, s = 0, t = 0;
    bool saved = false;             // sph_engine_save_state holds a copy
    double saved_time = 0.0;
    float saved_elapsed = 0.f;
};

struct sph_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<SceneInput> inputs;
    std::vector<std::vector<float>> storage;
    StepState state;
    bool finalized = false;
    StepMode mode = StepMode::Persistent;
    uint32_t grid = 0;
    sph::TuneChoice tuned{StepMode::Persistent, 0u, 0, 0, 0.f};
    bool tuned_from_cache = false;
};

#define API_CUDA_TRY(expr)                                                                     \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            sph::set_last_error(std::string(#expr) + ": " + cudaGetErrorString(e_));           \
            return e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;     \
        }                                                                                      \
    } while (0)

#define API_TRY(expr)                          \
    do {                                       \
        sph_status s_ = (expr);                \
        if (s_ != SPH_OK) return s_;           \
    } while (0)

static sph_status make_stream(int device, cudaStream_t* stream)
{
    int count = 0;
    API_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) {
        sph::set_last_error("no such CUDA device");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    API_CUDA_TRY(cudaSetDevice(device));
    API_CUDA_TRY(cudaStreamCreateWithFlags(stream, cudaStreamNonBlocking));
    return SPH_OK;
}

extern "C" {

SPH_API const char* sph_status_string(sph_status status)
{
    switch (status) {
    case SPH_OK: return "ok";
    case SPH_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SPH_ERR_NOT_INITIALIZED: return "engine not initialized";
    case SPH_ERR_CUDA: return "CUDA error";
    case SPH_ERR_OUT_OF_MEMORY: return "out of device memory";
    case SPH_ERR_DEVICE_TIMEOUT: return "bounded device wait expired";
    case SPH_ERR_CAPACITY: return "capacity exceeded";
    case SPH_ERR_BUDGET: return "HBM budget exceeded";
    case SPH_ERR_NOT_FOUND: return "not found";
    }
    return "unknown status";
}

SPH_API const char* sph_last_error(void) { return sph::last_error(); }

SPH_API const char* sph_engine_implementation_name(void) { return "CUDA-sm_103a"; }

// ---- engine -----------------------------------------------------------------

SPH_API sph_status sph_engine_create(sph_engine** out, int device)
{
    if (!out) return SPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cudaStream_t stream = nullptr;
    API_TRY(make_stream(device, &stream));
    sph_engine* e = new (std::nothrow) sph_engine();
    if (!e) { cudaStreamDestroy(stream); return SPH_ERR_OUT_OF_MEMORY; }
    e->device = device;
    e->stream = stream;
    *out = e;
    return SPH_OK;
}

SPH_API sph_status sph_engine_destroy(sph_engine* e)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    e->state.release();
    cudaStreamDestroy(e->stream);
    delete e;
    return SPH_OK;
}

SPH_API sph_status sph_engine_clear(sph_engine* e)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    API_CUDA_TRY(cudaSetDevice(e->device));
    API_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->state.drop_scenes();
    e->initialized = false;
    e->sim_time = 0.0;
    e->reorder_elapsed = 0.f;
    e->n = e->s = e->t = 0;
    e->accel_valid = false;
    e->saved = false;
    return SPH_OK;
}

SPH_API sph_status sph_engine_initialize(sph_engine* e, const sph_params* params, const float* dyn_pos,
                                         const float* dyn_vel, uint32_t n, const float* static_pos, uint32_t s,
                                         const float* triangles, uint32_t t, float reorder_time_interval)
{
    if (!e || !params) return SPH_ERR_INVALID_ARGUMENT;
    API_TRY(sph_engine_clear(e));
    SceneInput in;
    in.params = *params;
    in.pos = dyn_pos;
    in.vel = dyn_vel;
    in.n = n;
    in.spos = static_pos;
    in.s = s;
    in.tris = triangles;
    in.t = t;
    in.dt = 0.f;
    API_TRY(e->state.build(e->device, e->stream, {in}));
    e->n = n;
    e->s = s;
    e->t = t;
    e->reorder_interval = reorder_time_interval;
    e->initialized = true;
    return SPH_OK;
}

static sph_status engine_enqueue(sph_engine* e, float dt, uint32_t steps)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) {
        sph::set_last_error("Update called on an uninitialized engine");
        return SPH_ERR_NOT_INITIALIZED;
    }
    if (e->n == 0) return SPH_OK;
    API_CUDA_TRY(cudaSetDevice(e->device));
    // SimulationEngineCPU.cpp:441,452-454: one reorder decision per call, for
    // all of its steps; the elapsed time advances by dt per call
    API_TRY(e->state.set_reorder(0, e->reorder_elapsed > e->reorder_interval));
    API_TRY(e->state.set_dt(0, dt));
    API_TRY(e->state.enqueue_steps(steps, StepMode::Staged, e->record_accel, e->timing));
    e->reorder_elapsed += dt;
    if (e->reorder_elapsed > e->reorder_interval) e->reorder_elapsed = 0.f;
    e->sim_time += (double)dt * steps;
    e->accel_valid = e->record_accel;
    return SPH_OK;
}

SPH_API sph_status sph_engine_update_async(sph_engine* e, float dt, uint32_t steps)
{
    return engine_enqueue(e, dt, steps);
}

SPH_API sph_status sph_engine_synchronize(sph_engine* e)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.check_device_error();   // waits for the stream
}

SPH_API sph_status sph_engine_update(sph_engine* e, float dt, uint32_t steps)
{
    API_TRY(engine_enqueue(e, dt, steps));
    return sph_engine_synchronize(e);
}

SPH_API sph_status sph_engine_read_dynamic(sph_engine* e, sph_dynamic_particle* out)
{
    if (!e || (!out && e->n)) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.read_scene(0, out, nullptr);
}

SPH_API sph_status sph_engine_read_dynamic_buffer(sph_engine* e, sph_dynamic_particle* out)
{
    if (!e || (!out && e->n)) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.read_scene(0, out, nullptr, /*buffer_order=*/true);
}

SPH_API sph_status sph_engine_write_dynamic(sph_engine* e, const sph_dynamic_particle* in)
{
    if (!e || (!in && e->n)) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.write_scene(0, in);
}

SPH_API sph_status sph_engine_write_dynamic_async(sph_engine* e, const sph_dynamic_particle* in)
{
    if (!e || (!in && e->n)) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.write_scene(0, in, /*wait=*/false);
}

SPH_API sph_status sph_engine_read_static(sph_engine* e, sph_static_particle* out, uint32_t* bucket_starts)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.read_static(0, out, bucket_starts);
}

SPH_API sph_status sph_engine_read_buckets(sph_engine* e, uint32_t* bucket_starts, uint32_t* slot_ids)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.read_buckets(0, bucket_starts, slot_ids);
}

SPH_API sph_status sph_engine_simulation_time(sph_engine* e, double* seconds)
{
    if (!e || !seconds) return SPH_ERR_INVALID_ARGUMENT;
    *seconds = e->sim_time;
    return SPH_OK;
}

SPH_API sph_status sph_engine_count(sph_engine* e, int which, uint64_t* value)
{
    if (!e || !value) return SPH_ERR_INVALID_ARGUMENT;
    switch (which) {
    case 0: *value = e->n; break;
    case 1: *value = e->s; break;
    case 2: *value = 2ull * e->n; break;
    case 3: *value = e->t; break;
    default: return SPH_ERR_INVALID_ARGUMENT;
    }
    return SPH_OK;
}

SPH_API sph_status sph_engine_render(sph_engine* e, const sph_render_view* view,
                                     const sph_render_layer* dynamic_layer, const sph_render_layer* static_layer,
                                     uint8_t* rgba, float* depth)
{
    if (!e || !view) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    return e->state.render(*view, dynamic_layer, static_layer, rgba, depth);
}

SPH_API sph_status sph_debug_expire_wait(int device, uint32_t* status_bits)
{
    if (!status_bits) return SPH_ERR_INVALID_ARGUMENT;
    *status_bits = 0;
    return sph::scan_wait_probe(device, status_bits);
}

SPH_API sph_status sph_engine_set_exact(sph_engine* e, int exact)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    API_CUDA_TRY(cudaSetDevice(e->device));
    API_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->state.set_exact(exact != 0);
    return SPH_OK;
}

SPH_API sph_status sph_engine_record_acceleration(sph_engine* e, int on)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    e->record_accel = on != 0;
    if (!e->record_accel) e->accel_valid = false;
    return SPH_OK;
}

SPH_API sph_status sph_engine_read_acceleration(sph_engine* e, float* out)
{
    if (!e || (!out && e->n)) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    if (!e->accel_valid) {
        sph::set_last_error("no step was run with acceleration recording on");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (!e->n) return SPH_OK;
    API_CUDA_TRY(cudaSetDevice(e->device));
    std::vector<sph_dynamic_particle> scratch(e->n);
    return e->state.read_scene(0, scratch.data(), out);
}

SPH_API sph_status sph_engine_set_timing(sph_engine* e, int on)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    e->timing = on != 0;
    return SPH_OK;
}

SPH_API sph_status sph_engine_kernel_times(sph_engine* e, float* ms, int count)
{
    if (!e || !ms || count < 0) return SPH_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < count && k < 5; ++k) ms[k] = e->state.stage_ms()[k];
    return SPH_OK;
}

SPH_API sph_status sph_engine_neighbour_stats(sph_engine* e, sph_neighbour_stats* out)
{
    if (!e || !out) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(e->device));
    uint64_t v[sph::kNeighbourStats];
    API_TRY(e->state.neighbour_stats(v));
    out->particles = v[0];
    out->candidates = v[1];
    out->warp_slots = v[2];
    out->neighbours = v[3];
    out->static_neighbours = v[4];
    out->group_candidates = v[5];
    out->group_lane_slots = v[6];
    out->group_fallback = v[7];
    return SPH_OK;
}

SPH_API sph_status sph_engine_save_state(sph_engine* e)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized) {
        sph::set_last_error("sph_engine_save_state: no scene");
        return SPH_ERR_NOT_INITIALIZED;
    }
    API_CUDA_TRY(cudaSetDevice(e->device));
    if (e->n) API_TRY(e->state.save_state());
    e->saved = true;
    e->saved_time = e->sim_time;
    e->saved_elapsed = e->reorder_elapsed;
    return SPH_OK;
}

SPH_API sph_status sph_engine_restore_state(sph_engine* e)
{
    if (!e) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized || !e->saved) {
        sph::set_last_error("sph_engine_restore_state: nothing saved for this scene");
        return SPH_ERR_NOT_INITIALIZED;
    }
    API_CUDA_TRY(cudaSetDevice(e->device));
    if (e->n) API_TRY(e->state.restore_state());
    e->sim_time = e->saved_time;
    e->reorder_elapsed = e->saved_elapsed;
    e->accel_valid = false;
    return SPH_OK;
}

SPH_API sph_status sph_engine_get_stream(sph_engine* e, void** stream)
{
    if (!e || !stream) return SPH_ERR_INVALID_ARGUMENT;
    *stream = (void*)e->stream;
    return SPH_OK;
}

// ---- the counting sort on its own ---------------------------------------------

SPH_API sph_status sph_cell_sort(int device, const float* pos, uint32_t n, float h, uint32_t buckets, uint32_t* keys,
                                 uint32_t* counts, uint32_t* starts, uint32_t* order)
{
    if ((!pos && n) || buckets == 0 || !(h > 0.f)) return SPH_ERR_INVALID_ARGUMENT;
    if (n > sph::kMaxParticles || buckets > (1u << 31)) return SPH_ERR_CAPACITY;
    cudaStream_t stream = nullptr;
    API_TRY(make_stream(device, &stream));
    sph_status st;
    {
        StepState state;
        SceneInput in;
        in.params.max_interaction_distance = h;
        in.params.gas_constant = 1.f;
        in.pos = pos;
        in.n = n;
        in.buckets = buckets;
        st = state.build(device, stream, {in});
        if (st == SPH_OK) st = state.read_sort(keys, counts, starts, order);
    }
    cudaStreamDestroy(stream);
    return st;
}

// ---- batch ---------------------------------------------------------------------

SPH_API sph_status sph_batch_create(sph_batch** out, int device)
{
    if (!out) return SPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cudaStream_t stream = nullptr;
    API_TRY(make_stream(device, &stream));
    sph_batch* b = new (std::nothrow) sph_batch();
    if (!b) { cudaStreamDestroy(stream); return SPH_ERR_OUT_OF_MEMORY; }
    b->device = device;
    b->stream = stream;
    *out = b;
    return SPH_OK;
}

SPH_API sph_status sph_batch_destroy(sph_batch* b)
{
    if (!b) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    b->state.release();
    cudaStreamDestroy(b->stream);
    delete b;
    return SPH_OK;
}

SPH_API sph_status sph_batch_add_scene(sph_batch* b, const sph_params* params, const float* dyn_pos,
                                       const float* dyn_vel, uint32_t n, const float* static_pos, uint32_t s,
                                       const float* triangles, uint32_t t, float dt, uint32_t* scene_id)
{
    if (!b || !params) return SPH_ERR_INVALID_ARGUMENT;
    if (b->finalized) {
        sph::set_last_error("batch already finalized");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SceneInput in;
    in.params = *params;
    in.n = n;
    in.s = s;
    in.t = t;
    in.dt = dt;
    in.pos = dyn_pos;
    in.vel = dyn_vel;
    in.spos = static_pos;
    in.tris = triangles;
    API_TRY(sph::validate_scene(in));
    auto keep = [&](const float* p, size_t cnt) -> const float* {
        if (!p || !cnt) return nullptr;
        b->storage.emplace_back(p, p + cnt);
        return b->storage.back().data();
    };
    in.pos = keep(dyn_pos, 3ull * n);
    in.vel = keep(dyn_vel, 3ull * n);
    in.spos = keep(static_pos, 3ull * s);
    in.tris = keep(triangles, 9ull * t);
    if (scene_id) *scene_id = (uint32_t)b->inputs.size();
    b->inputs.push_back(in);
    return SPH_OK;
}

SPH_API sph_status sph_batch_finalize(sph_batch* b)
{
    if (!b) return SPH_ERR_INVALID_ARGUMENT;
    if (b->finalized) return SPH_OK;
    API_CUDA_TRY(cudaSetDevice(b->device));
    API_TRY(b->state.build(b->device, b->stream, b->inputs));
    b->storage.clear();
    for (auto& in : b->inputs) { in.pos = in.vel = in.spos = in.tris = nullptr; }
    API_TRY(b->state.persistent_grid(&b->grid));
    b->finalized = true;
    return SPH_OK;
}

static void fill_config(const StepState& st, const sph::TuneChoice& c, bool from_cache, uint32_t grid,
                        sph_launch_config* out)
{
    if (!out) return;
    out->mode = c.mode == StepMode::Persistent ? 0 : 1;
    out->persistent_ctas = c.mode == StepMode::Persistent ? grid : 0u;
    out->density_threads = sph::kShapeInfo[st.density_shape()].threads;
    out->density_min_ctas = sph::kShapeInfo[st.density_shape()].min_ctas;
    out->force_threads = sph::kShapeInfo[st.force_shape()].threads;
    out->force_min_ctas = sph::kShapeInfo[st.force_shape()].min_ctas;
    out->ms_per_step = c.ms;
    out->from_cache = from_cache ? 1 : 0;
    out->density_walk = sph::kShapeInfo[st.density_shape()].slot_walk;
}

// The launch autotuner over the batch (StepState::autotune, staged shapes
// and persistent grid sizes); the choice is kept for sph_batch_step.
SPH_API sph_status sph_batch_autotune(sph_batch* b, uint32_t trial_steps, int* mode_out, uint32_t* grid_out,
                                      float* ms_per_step_out)
{
    if (!b || trial_steps == 0) return SPH_ERR_INVALID_ARGUMENT;
    if (!b->finalized) API_TRY(sph_batch_finalize(b));
    API_CUDA_TRY(cudaSetDevice(b->device));
    sph::TuneChoice c{};
    bool cached = false;
    API_TRY(b->state.autotune(trial_steps, true, &c, &cached));
    b->mode = c.mode;
    b->tuned = c;
    b->tuned_from_cache = cached;
    API_TRY(b->state.persistent_grid(&b->grid));
    if (mode_out) *mode_out = c.mode == StepMode::Persistent ? 0 : 1;
    if (grid_out) *grid_out = c.mode == StepMode::Persistent ? b->grid : 0;
    if (ms_per_step_out) *ms_per_step_out = c.ms;
    return SPH_OK;
}

SPH_API sph_status sph_batch_launch_config(sph_batch* b, sph_launch_config* out)
{
    if (!b || !out) return SPH_ERR_INVALID_ARGUMENT;
    if (!b->finalized) API_TRY(sph_batch_finalize(b));
    API_CUDA_TRY(cudaSetDevice(b->device));
    API_TRY(b->state.persistent_grid(&b->grid));
    sph::TuneChoice c = b->tuned;
    c.mode = b->mode;
    fill_config(b->state, c, b->tuned_from_cache, b->grid, out);
    return SPH_OK;
}

SPH_API sph_status sph_engine_set_launch_shapes(sph_engine* e, int density_shape, int force_shape)
{
    if (!e || density_shape < 0 || density_shape >= sph::kShapeCount || force_shape < 0 ||
        force_shape >= sph::kForceShapeCount)
        return SPH_ERR_INVALID_ARGUMENT;
    API_CUDA_TRY(cudaSetDevice(e->device));
    API_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->state.set_shapes(density_shape, force_shape);
    return SPH_OK;
}

SPH_API sph_status sph_engine_autotune(sph_engine* e, uint32_t trial_steps, sph_launch_config* out)
{
    if (!e || trial_steps == 0) return SPH_ERR_INVALID_ARGUMENT;
    if (!e->initialized || e->n == 0) {
        sph::set_last_error("sph_engine_autotune: no scene");
        return SPH_ERR_NOT_INITIALIZED;
    }
    API_CUDA_TRY(cudaSetDevice(e->device));
    sph::TuneChoice c{};
    bool cached = false;
    e->saved = false;                   // the trials use the engine's checkpoint slot
    // the trials run with this scene's reorder flag and dt as they stand
    API_TRY(e->state.autotune(trial_steps, false, &c, &cached));
    fill_config(e->state, c, cached, 0u, out);
    return SPH_OK;
}

SPH_API sph_status sph_batch_set_mode(sph_batch* b, int mode)
{
    if (!b || (mode != 0 && mode != 1)) return SPH_ERR_INVALID_ARGUMENT;
    b->mode = mode == 0 ? StepMode::Persistent : StepMode::Staged;
    return SPH_OK;
}

SPH_API sph_status sph_batch_set_exact(sph_batch* b, int exact)
{
    if (!b) return SPH_ERR_INVALID_ARGUMENT;
    API_CUDA_TRY(cudaSetDevice(b->device));
    API_CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->state.set_exact(exact != 0);
    return SPH_OK;
}

SPH_API sph_status sph_batch_step(sph_batch* b, uint32_t steps)
{
    if (!b) return SPH_ERR_INVALID_ARGUMENT;
    if (!b->finalized) API_TRY(sph_batch_finalize(b));
    API_CUDA_TRY(cudaSetDevice(b->device));
    API_TRY(b->state.enqueue_steps(steps, b->mode, false, false));
    return b->state.check_device_error();   // waits for the stream
}

SPH_API sph_status sph_batch_read_scene(sph_batch* b, uint32_t scene_id, sph_dynamic_particle* out)
{
    if (!b || !out) return SPH_ERR_INVALID_ARGUMENT;
    if (!b->finalized) return SPH_ERR_NOT_INITIALIZED;
    API_CUDA_TRY(cudaSetDevice(b->device));
    return b->state.read_scene(scene_id, out, nullptr);
}

SPH_API sph_status sph_batch_info(sph_batch* b, uint64_t* total_particles, uint32_t* grid_ctas,
                                  uint32_t* threads_per_cta)
{
    if (!b) return SPH_ERR_INVALID_ARGUMENT;
    if (total_particles) {
        uint64_t t = 0;
        for (auto& in : b->inputs) t += in.n;
        *total_particles = t;
    }
    if (grid_ctas) *grid_ctas = b->grid;
    if (threads_per_cta) *threads_per_cta = sph::kTileThreads;
    return SPH_OK;
}

}  // extern "C"
