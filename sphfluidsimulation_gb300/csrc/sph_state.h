// sph_state.h -- device state of one or more SPH scenes and the launches
// that advance it.  Used by the single-scene engine, the batch and the
// server behind the C ABI in include/sph_gb300.h.
#pragma once
#include <cmath>
#include <string>
#include <vector>

#include "sph_gb300.h"
#include "sph_kernels.cuh"

namespace sph {

constexpr uint64_t kMaxParticles = 1ull << 30;

struct SortArgs {
    const Tile* tiles;
    const SceneDesc* scenes;
    const float4* pos_src;
    const float4* vel_src;
    float4* pos_dst;
    float4* vel_dst;
    uint32_t* key;
    uint32_t* arrival;
    uint32_t* ptag;             // scatter slot -> tag
    const uint32_t* tag_src;    // tag per source slot; null: the source slot itself
    uint32_t* tag_dst;          // tag per sorted slot (unused with kTagNone)
    uint32_t assign;            // TagAssign
    const float4* accel_src;    // recorded acceleration per source slot, moved along (or null)
    float4* accel_dst;
    const uint32_t* tag_keep;   // kTagKeep: tag per source slot when tag_src is only a ranking key
    uint32_t* count;
    uint32_t* start;
    uint32_t* err;
    uint32_t* nonfinite_set;     // hash + count marks a non-finite position here (or null)
    uint32_t* nonfinite_rotate;  // the step's gather moves [1] to [0] and clears [1] (or null)
};

// One scene as the caller hands it over (host pointers, caller's order).
struct SceneInput {
    sph_params params{};
    const float* pos = nullptr;    // n x 3
    const float* vel = nullptr;    // n x 3 or null
    uint32_t n = 0;
    const float* spos = nullptr;   // s x 3
    uint32_t s = 0;
    const float* tris = nullptr;   // t x 9
    uint32_t t = 0;
    float dt = 0.f;
    uint32_t buckets = 0;          // dynamic bucket count; 0 = 2n (SimulationEngineCPU.cpp:486)
};

enum class StepMode { Staged = 0, Persistent = 1 };

// Launch shapes of the two neighbour passes in the default arithmetic
// (sph_shapes.cu): threads per CTA, the register bound's resident CTAs per
// SM and, for density, the walk (0 the group walk, 1 the per-slot walk).
// Shape 0 is the default kernel; every shape computes the same bits.  The
// force pass has the first kForceShapeCount shapes.
constexpr int kShapeCount = 6;
constexpr int kNeighbourStats = 8;     // counters of k_neighbour_stats
constexpr int kForceShapeCount = 5;
struct ShapeInfo {
    int threads;
    int min_ctas;
    int slot_walk;
};
constexpr ShapeInfo kShapeInfo[kShapeCount] = {
    {kTileThreads, SPH_DENSITY_MIN_CTAS, 0}, {64, 14, 0}, {256, 3, 0}, {128, 6, 0}, {128, 8, 0},
    {kTileThreads, SPH_DENSITY_MIN_CTAS, 1}};
cudaError_t launch_shaped(int shape, bool density, const StepArgs& a, cudaStream_t s);

// One configuration of the step: staged (with the two passes' shapes) or
// persistent (with its grid), and its measured time per step.
struct TuneChoice {
    StepMode mode;
    uint32_t ctas;          // persistent grid, 0 = the occupancy limit
    int density_shape;
    int force_shape;
    float ms;
};

void set_last_error(const std::string& s);
const char* last_error();

#define CUDA_TRY(expr)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            set_last_error(std::string(#expr) + ": " + cudaGetErrorString(e_));                    \
            return e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;          \
        }                                                                                           \
    } while (0)

template <typename T>
inline sph_status dev_alloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    CUDA_TRY(cudaMalloc((void**)p, sizeof(T) * count));
    return SPH_OK;
}

sph_status validate_scene(const SceneInput& in);
// Makes the scan's bounded look-back expire on purpose (see sph_step.cu).
sph_status scan_wait_probe(int device, uint32_t* status_bits);
// Physics constants and sizes of a scene (offsets left zero).
SceneDesc scene_desc_for(const SceneInput& in);

class StepState {
public:
    StepState() = default;
    StepState(const StepState&) = delete;
    StepState& operator=(const StepState&) = delete;
    ~StepState();

    // Lays the scenes out back to back, allocates, uploads and sorts them.
    sph_status build(int device, cudaStream_t stream, const std::vector<SceneInput>& inputs);
    void release();              // drop_scenes() + free_device_arrays()
    void drop_scenes();          // forget the scenes, keep the device arrays
    void free_device_arrays();

    // Queues `steps` steps of every scene.  Staged mode replays a captured
    // CUDA graph of the five stage launches; persistent mode issues one
    // cooperative launch per step.  `timed` records per-stage events.
    sph_status enqueue_steps(uint32_t steps, StepMode mode, bool record_accel, bool timed);
    sph_status check_device_error();

    sph_status set_dt(uint32_t scene, float dt);
    // Whether the steps queued next renumber the scene's buffer tags, as a
    // reordering Update of the reference does (SimulationEngineCPU.cpp:441).
    sph_status set_reorder(uint32_t scene, bool reorder);
    // Neighbour-pass arithmetic: false fused/fast, true the reference's own.
    void set_exact(bool exact)
    {
        if (exact != exact_) drop_graphs();
        if (exact != exact_) grid_cache_ = 0;
        exact_ = exact;
    }
    bool exact() const { return exact_; }
    // Caller's order, or with buffer_order the reference's buffer order (by tag).
    sph_status read_scene(uint32_t scene, sph_dynamic_particle* out, float* accel_out, bool buffer_order = false);
    // wait = false leaves the upload and re-sort queued on the stream (the
    // caller keeps `in` unchanged until the next synchronising call)
    sph_status write_scene(uint32_t scene, const sph_dynamic_particle* in, bool wait = true);
    sph_status read_static(uint32_t scene, sph_static_particle* out, uint32_t* bucket_starts);
    sph_status read_buckets(uint32_t scene, uint32_t* bucket_starts, uint32_t* slot_ids);
    // particles, candidates, warp candidate slots, dynamic and static
    // neighbours within h, summed over all scenes (k_neighbour_stats)
    sph_status neighbour_stats(uint64_t out[kNeighbourStats]);
    sph_status persistent_grid(uint32_t* grid);
    // Outputs of the initial sort of scene 0 (see sph_cell_sort).
    sph_status read_sort(uint32_t* keys, uint32_t* counts, uint32_t* starts, uint32_t* order);

    // ---- arena mode (server): fixed-capacity arrays, each scene occupies
    // ranges of the slot / bucket / static index spaces chosen by the caller.
    sph_status init_arena(int device, cudaStream_t stream, uint32_t cap_n, uint32_t cap_q, uint32_t cap_s,
                          uint32_t cap_sq, uint32_t cap_sf, uint32_t cap_sbm, uint32_t max_scenes);
    // Grows every array to at least the given capacities, keeping contents.
    sph_status grow_arena(uint32_t cap_n, uint32_t cap_q, uint32_t cap_s, uint32_t cap_sq, uint32_t cap_sf,
                          uint32_t cap_sbm);
    // Uploads one scene into its ranges (d's offsets) and sorts it alone.
    // With sync = false the work is only queued (check_device_error later).
    // With host_direct the kernels read the scene's particles from the
    // caller's (pageable) arrays themselves, which must stay valid until the
    // work completes (GPUs with pageable memory access only).
    sph_status admit_scene(const SceneDesc& d, const SceneInput& in, bool sync = true, bool host_direct = false);
    // Queues a readback of one scene into host memory the GPU writes itself.
    sph_status read_scene_async(uint32_t scene, sph_dynamic_particle* out);
    // Replaces the set of scenes the step advances (table, tiles, scan range).
    sph_status set_active(const std::vector<SceneDesc>& descs);
    uint32_t cap_n() const { return cap_n_; }
    uint32_t cap_q() const { return cap_q_; }
    uint32_t cap_s() const { return cap_s_; }
    uint32_t cap_sq() const { return cap_sq_; }
    uint32_t cap_sf() const { return cap_sf_; }
    uint32_t cap_sbm() const { return cap_sbm_; }

    // Headless particle splats of scene 0 (see sph_engine_render).
    sph_status render(const sph_render_view& view, const sph_render_layer* dyn, const sph_render_layer* stat,
                      uint8_t* rgba_out, float* depth_out);

    // Copies the state a step reads (sorted particles and the bucket table)
    // aside and back, so trial steps leave the simulation where it was.
    sph_status save_state();
    sph_status restore_state();
    // Occupancy-limited CTAs per SM of the persistent step kernel.
    sph_status persistent_capacity(uint32_t* sms, uint32_t* per_sm);

    // Launch shapes of the staged step's density and force passes (default
    // arithmetic, accelerations not recorded); 0 = the default kernels.
    void set_shapes(int density, int force)
    {
        if (density != density_shape_ || force != force_shape_) drop_graphs();
        density_shape_ = density;
        force_shape_ = force;
    }
    int density_shape() const { return density_shape_; }
    int force_shape() const { return force_shape_; }

    // The launch autotuner (sph_tune.cu): times the staged step under each
    // launch shape of the two neighbour passes and, with allow_persistent,
    // the persistent step at each grid size, on a saved copy of the state
    // (which replaces any earlier save_state copy); applies and returns the
    // fastest.  Choices are cached per GPU and size class.
    sph_status autotune(uint32_t trial_steps, bool allow_persistent, TuneChoice* out, bool* from_cache);
    void apply_choice(const TuneChoice& c);

    const float* stage_ms() const { return stage_ms_; }
    void set_persistent_ctas(uint32_t c)
    {
        persistent_ctas_ = c;
        grid_cache_ = 0;
    }

    std::vector<SceneDesc> scenes;
    std::vector<Tile> tiles, stiles;
    uint32_t total_n = 0, total_s = 0, total_t = 0;
    uint32_t scan_len = 0, sscan_len = 0, sfscan_len = 0;

    // device arrays
    SceneDesc* d_scenes = nullptr;
    SceneDesc* d_sscenes = nullptr;
    Tile* d_tiles = nullptr;
    Tile* d_stiles = nullptr;
    float4 *pos = nullptr, *vel = nullptr, *pos_tmp = nullptr, *vel_tmp = nullptr;
    uint32_t *key = nullptr, *arrival = nullptr, *ptag = nullptr, *count = nullptr, *start = nullptr;
    uint32_t* tag = nullptr;       // buffer tag per sorted slot
    uint32_t* tag_io = nullptr;    // tags in caller's order while a write re-sorts
    uint32_t* rank_io = nullptr;   // ~(slot before the write) in caller's order: the write's ranking key
    unsigned long long* scan_status = nullptr;
    uint32_t* scan_ticket = nullptr;
    uint32_t* err = nullptr;
    uint32_t* bar = nullptr;
    // [0]: some current position is not finite (read by the walks);
    // [1]: the same for the positions the force pass is writing
    uint32_t* nonfinite = nullptr;
    float4* spos = nullptr;        // statics sorted by the neighbour-pass table
    uint32_t* sstart = nullptr;
    float4* spos_ref = nullptr;    // statics sorted by the reference's s-bucket table
    uint32_t* sstart_ref = nullptr;
    uint32_t* nbr = nullptr;       // neighbour lists, [kMaxNbr][cap_n]
    uint32_t* snbr = nullptr;      // [kMaxSNbr][cap_n]
    uint32_t* ncount = nullptr;
    uint32_t* tile_overflow = nullptr;
    uint32_t* sbitmap = nullptr;   // static-presence bitmaps (words)
    SceneDesc* d_sfscenes = nullptr;
    float* tris = nullptr;
    uint32_t* tri_cells = nullptr;  // triangle cells of every scene with triangles
    uint32_t* tri_list = nullptr;
    float4* accel = nullptr;       // recorded acceleration per sorted slot
    float4* accel_tmp = nullptr;   // as the force pass writes it (per tmp slot)
    float4* accel_io = nullptr;
    float4* staging = nullptr;

private:
    // sort kinds: 0 dynamic, 1 statics by the reference's table, 2 statics by
    // the neighbour-pass table
    sph_status enqueue_load(const float4* src, bool statics);
    sph_status enqueue_sort(int kind, bool keep_tags = false);
    sph_status enqueue_scan(uint32_t* cnt, uint32_t* out, uint32_t len, bool cleared = false);
    sph_status alloc_arrays(uint32_t cap_n, uint32_t cap_q, uint32_t cap_s, uint32_t cap_sq, uint32_t cap_sf,
                            uint32_t cap_sbm, uint32_t cap_t, uint32_t max_scenes, uint32_t max_tiles);
    sph_status zero_state_arrays();
    sph_status enqueue_step_staged(bool record_accel, bool timed);
    sph_status enqueue_step_persistent();
    sph_status ensure_events();
    SortArgs sort_args(int kind) const;
    template <bool kExact>
    sph_status launch_step_staged(bool record_accel, bool timed);
    unsigned overflow_grid(unsigned tiles_n);
    StepArgs step_args() const;
    std::string tune_key(bool allow_persistent) const;

    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;        // one staged step
    cudaGraphExec_t graph_timed_ = nullptr;  // the same with event records between the stages
    void drop_graphs()
    {
        if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
        if (graph_timed_) { cudaGraphExecDestroy(graph_timed_); graph_timed_ = nullptr; }
    }
    cudaEvent_t events_[6] = {};
    float stage_ms_[5] = {};
    uint32_t persistent_ctas_ = 0;
    int density_shape_ = 0, force_shape_ = 0;
    bool exact_ = false;
    uint32_t sm_count_ = 0;
    uint32_t grid_cache_ = 0;
    uint32_t cap_n_ = 0, cap_q_ = 0, cap_s_ = 0, cap_sq_ = 0, cap_sf_ = 0, cap_sbm_ = 0, cap_t_ = 0, max_scenes_ = 0,
             max_tiles_ = 0;
    std::vector<uint32_t> tile_first_;     // first tile of each scene
    Tile* d_tmp_tiles_ = nullptr;          // tiles of a scene being admitted
    uint32_t* d_tile_first_ = nullptr;     // arena: first tile of each active scene (+ the total)
    float4* saved_pos_ = nullptr;          // save_state() copies
    float4* saved_vel_ = nullptr;
    uint32_t* saved_start_ = nullptr;
    uint32_t* saved_tag_ = nullptr;
    uint32_t saved_nonfinite_[2] = {0u, 0u};
    uint32_t* err_host_ = nullptr;                // pinned copy of the status word
    unsigned long long* render_zkey_ = nullptr;   // render targets, kept between frames
    uchar4* render_rgba_ = nullptr;
    float* render_depth_ = nullptr;
    size_t render_pixels_ = 0;
    SceneDesc* d_tmp_scene_ = nullptr;     // its dynamic and two static views
};

}  // namespace sph
