// sph_step.cu -- kernels of the SPH step and the device-state object that
// launches them (one scene or many).
//
// Per step, over every tile of every scene:
//   density  (vel.w = pressure)                      reference SF:358-501
//   force    (tmp = integrated particles, key, count) reference SF:503-656
//   scan     (start = exclusive scan of count)        reference SF:227-294 / ECPU:245-253
//   scatter  (ptag[start+arrival] = buffer tag)       reference SF:346-356
//   gather   (rank by tag, tmp -> sorted state)       reference SF:332-345
// either as five launches (captured once in a CUDA graph) or as one
// persistent cooperative launch with four bounded grid barriers.
#include "sph_state.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace sph {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kTileThreads) k_hash_count(SortArgs a)
{
    hash_count_tile(a.tiles[blockIdx.x], a.scenes, a.pos_src, a.key, a.arrival, a.count, a.nonfinite_set);
}

__global__ void __launch_bounds__(kScanThreads) k_scan(uint32_t* count, uint32_t* start, uint32_t len,
                                                       unsigned long long* status, uint32_t* ticket, uint32_t* err)
{
    __shared__ ScanSmem sm;
    if (threadIdx.x == 0) sm.tile = atomicAdd(ticket, 1u);
    __syncthreads();
    scan_tile(sm.tile, count, start, len, status, err, sm);
}

__global__ void __launch_bounds__(kTileThreads) k_scatter(SortArgs a)
{
    scatter_tile(a.tiles[blockIdx.x], a.scenes, a.key, a.arrival, a.start, a.tag_src, a.ptag, a.err);
}

__global__ void __launch_bounds__(kTileThreads) k_gather(SortArgs a)
{
    gather_tile(a.tiles[blockIdx.x], a.scenes, a.key, a.arrival, a.ptag, a.start, a.pos_src, a.vel_src,
                a.pos_dst, a.vel_dst, a.tag_dst, a.assign, a.err, a.accel_src, a.accel_dst, a.tag_keep);
    if (a.nonfinite_rotate && blockIdx.x == 0 && threadIdx.x == 0) {   // the force pass has finished
        a.nonfinite_rotate[0] = a.nonfinite_rotate[1];
        a.nonfinite_rotate[1] = 0u;
    }
}

template <bool kExact>
__global__ void __launch_bounds__(kDensityThreads, SPH_DENSITY_MIN_CTAS) k_density(StepArgs a)
{
    __shared__ __align__(16) GroupSmem gsm[kDensityThreads / 32];
    density_group_tile<kExact>(blockIdx.x, a.tiles[blockIdx.x], threadIdx.x, a.scenes, a.pos, a.vel, a.start,
                               static_tables(a), nbr_args(a), gsm[threadIdx.x >> 5]);
}

template <bool kRecord, bool kExact>
__global__ void __launch_bounds__(kTileThreads, SPH_FORCE_MIN_CTAS) k_force(StepArgs a)
{
    force_tile<kRecord, kExact>(a.tiles[blockIdx.x], a.scenes, a.pos, a.vel, a.tag, static_tables(a), triangle_mesh(a),
                                nbr_args(a), force_out(a));
}

// Particles whose neighbour list overflowed.  A grid of a few CTAs per SM
// walks the per-tile flags the density pass set, so a step without overflow
// costs one flag read per tile.  It also clears the look-back state of the
// scan that follows it in the step (the previous scan finished long before).
template <bool kRecord, bool kExact>
__global__ void __launch_bounds__(kTileThreads) k_force_overflow(StepArgs a)
{
    const uint32_t scan_tiles = (a.scan_len + kScanTile - 1) / kScanTile;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < scan_tiles; t += gridDim.x * blockDim.x)
        a.scan_status[t] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.scan_ticket = 0u;
    for (uint32_t t = blockIdx.x; t < a.num_tiles; t += gridDim.x) {
        if (a.tile_overflow[t] == 0u) continue;                  // the same for the whole CTA
        force_overflow_tile<kRecord, kExact>(a.tiles[t], a.scenes, a.pos, a.vel, a.tag, a.start,
                                             static_tables(a), triangle_mesh(a), nbr_args(a), force_out(a));
        __syncthreads();
        if (threadIdx.x == 0) a.tile_overflow[t] = 0u;            // every thread has read the flag
    }
}

// Neighbour statistics of the current state (a measurement, run outside the
// step): out[0] particles; out[1] dynamic candidates the per-slot density
// walk tests; out[2] the candidate slots the warps spend on them (a cell
// costs a warp its largest bucket, so out[2] / out[1] is the divergence
// overhead); out[3] dynamic neighbours within h (each ordered pair once);
// out[4] static particles within h of a dynamic one; out[5] candidates the
// group walk tests its homes against (every member of the 27 buckets);
// out[6] the lane-slots it spends (32 per register slot and home); out[7]
// slots it leaves to the per-slot walk (crowded cells, non-finite slots).
__global__ void __launch_bounds__(kTileThreads) k_neighbour_stats(StepArgs a, unsigned long long* out)
{
    const Tile& tile = a.tiles[blockIdx.x];
    const SceneDesc& sc = a.scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    const bool valid = i < tile.end;
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    unsigned long long v[kNeighbourStats] = {valid ? 1ull : 0ull};
    if (valid) {
        const float4 p = a.pos[i];
        const Walk w = make_walk<false>(sc, p, a.sbitmap, a.nonfinite[0] != 0u);
        walk_neighbours_cells<false>(
            sc, i, p, w, a.pos, a.start, static_tables(a),
            [&](uint32_t, const float4&, float) { ++v[3]; },
            [&](uint32_t, const float4&, float) { ++v[4]; },
            [&](uint32_t m) {               // every valid lane, 27 times, in step
                v[1] += m;
                v[2] += __reduce_max_sync(mask, m);
            });
        // the group walk: every member of the 27 buckets (density_group_tile)
        const uint32_t delta = sc.p_off - __ldg(a.start + sc.q_off);
        uint32_t total = 0;
        for (int k = 0; k < 27; ++k) {
            const uint32_t bk = sc.q_off + fast_mod(neighbour_hash(w.nb, k / 9, (k / 3) % 3, k % 3), sc.fm_b);
            const uint32_t beg = max(__ldg(a.start + bk) + delta, sc.p_off);
            const uint32_t end = min(__ldg(a.start + bk + 1) + delta, sc.p_off + sc.n);
            total += end > beg ? end - beg : 0u;
        }
        if (finite3(p) && total <= kGroupSlots * 32u) {
            v[5] = total;
            v[6] = 32ull * ((total + 31u) / 32u);
        } else {
            v[7] = 1;
        }
    }
#pragma unroll
    for (int k = 0; k < kNeighbourStats; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if ((threadIdx.x & 31u) == 0u && mask)
        for (int k = 0; k < kNeighbourStats; ++k) atomicAdd(out + k, v[k]);
}

// Bounded grid barrier for the persistent kernel (all CTAs co-resident by
// cooperative launch).  Sense by generation counter; on expiry the error word
// is set and the CTA proceeds, so the launch always terminates.
__device__ __forceinline__ void grid_barrier(uint32_t* count, uint32_t* gen, uint32_t* err)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t g0 = *(volatile uint32_t*)gen;
        __threadfence();
        if (atomicAdd(count, 1u) == gridDim.x - 1u) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            uint32_t spins = 0;
            while (*(volatile uint32_t*)gen == g0) {
                if (++spins > kSpinLimit) { atomicOr(err, DEV_ERR_BARRIER_TIMEOUT); break; }
                __nanosleep(spins < 64 ? 32 : 256);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// One whole step in one launch: density, force, scan, scatter, gather with a
// grid barrier between stages.  Tiles are taken grid-stride; scan tiles are
// taken in increasing order per CTA, so every look-back waits only on a tile
// a co-resident CTA reaches first.
template <bool kExact>
__global__ void __launch_bounds__(kTileThreads) k_step_persistent(StepArgs a, uint32_t scan_tiles)
{
    __shared__ ScanSmem sm;
    __shared__ __align__(16) GroupSmem gsm[kTileThreads / 32];
    // the previous scan (any launch before this one) is complete: clear its
    // tile status so this step's look-back starts from empty
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < scan_tiles; t += gridDim.x * blockDim.x)
        a.scan_status[t] = 0ull;
    const NbrArgs nl = nbr_args(a);
    const StaticTables st = static_tables(a);
    const ForceOut fo = force_out(a);
    const TriangleMesh tm = triangle_mesh(a);
    for (uint32_t t = blockIdx.x; t < a.num_tiles; t += gridDim.x)
        density_group_tile<kExact>(t, a.tiles[t], threadIdx.x, a.scenes, a.pos, a.vel, a.start, st, nl,
                                   gsm[threadIdx.x >> 5]);
    grid_barrier(a.bar_count, a.bar_gen, a.err);
    for (uint32_t t = blockIdx.x; t < a.num_tiles; t += gridDim.x) {
        force_tile<false, kExact>(a.tiles[t], a.scenes, a.pos, a.vel, a.tag, st, tm, nl, fo);
        if (a.tile_overflow[t]) {
            force_overflow_tile<false, kExact>(a.tiles[t], a.scenes, a.pos, a.vel, a.tag, a.start, st, tm, nl, fo);
            __syncthreads();
            if (threadIdx.x == 0) a.tile_overflow[t] = 0u;
        }
    }
    grid_barrier(a.bar_count, a.bar_gen, a.err);
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // every walk of this step has read [0]
        a.nonfinite[0] = a.nonfinite[1];
        a.nonfinite[1] = 0u;
    }
    for (uint32_t t = blockIdx.x; t < scan_tiles; t += gridDim.x)
        scan_tile(t, a.count, a.start, a.scan_len, a.scan_status, a.err, sm);
    grid_barrier(a.bar_count, a.bar_gen, a.err);
    for (uint32_t t = blockIdx.x; t < a.num_tiles; t += gridDim.x)
        scatter_tile(a.tiles[t], a.scenes, a.key, a.arrival, a.start, a.tag, a.ptag, a.err);
    grid_barrier(a.bar_count, a.bar_gen, a.err);
    for (uint32_t t = blockIdx.x; t < a.num_tiles; t += gridDim.x)
        gather_tile(a.tiles[t], a.scenes, a.key, a.arrival, a.ptag, a.start, a.pos_tmp, a.vel_tmp, a.pos, a.vel,
                    a.tag, kTagStep, a.err);
}

__global__ void __launch_bounds__(kTileThreads) k_static_bitmap(const Tile* tiles, const SceneDesc* scenes,
                                                                const float4* spos, uint32_t* sbitmap)
{
    static_bitmap_tile(tiles[blockIdx.x], scenes, spos, sbitmap);
}

// Readback: sorted slot i -> caller's order (or, with by_tag, the reference's
// buffer order), in the reference's 32-byte layout (Particles.h:9-17); hash =
// key of the position (SF:644-645).  Optionally the acceleration and the
// buffer tag move along.
__global__ void __launch_bounds__(kTileThreads) k_unsort(const Tile* tiles, const SceneDesc* scenes, const float4* pos,
                                                         const float4* vel, float4* out, const float4* accel_in,
                                                         float4* accel_out, const uint32_t* tag_in, uint32_t* tag_out,
                                                         int by_tag, uint32_t* rank_out = nullptr, uint32_t out_origin = 0)
{
    const Tile tile = tiles[blockIdx.x];
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    if (i >= tile.end) return;
    const float4 p = pos[i];
    const uint32_t id = by_tag ? tag_in[i] : __float_as_uint(p.w);
    if (id >= sc.n) return;
    const uint32_t o = sc.p_off + id;
    if (tag_out) tag_out[o] = tag_in[i];
    if (rank_out) rank_out[o] = ~i;   // larger for earlier slots: ranking by it keeps the order
    if (!out) return;   // tags only
    const float4 v = vel[i];
    const uint32_t key = fast_mod(cell_hash(p.x, p.y, p.z, sc.h), sc.fm_b);
    out[2 * (size_t)(o - out_origin)] = make_float4(p.x, p.y, p.z, v.w);
    out[2 * (size_t)(o - out_origin) + 1] = make_float4(v.x, v.y, v.z, __uint_as_float(key));
    if (accel_in) accel_out[o] = accel_in[i];
}

// Upload staging (caller's order, the reference's 32-byte records as float4
// pairs: position + pressure, velocity + hash) -> unsorted tmp arrays with
// the input index in pos.w and the record's pressure in vel.w, which a
// LockWrite-style upload keeps until the next density pass.
// Dynamic particles carry their input index in w; static particles carry
// the Morton code of their cell, which the neighbour passes compare against
// the cell being visited.
__global__ void __launch_bounds__(kTileThreads) k_load(const Tile* tiles, const SceneDesc* scenes, const float4* in,
                                                       float4* pos_tmp, float4* vel_tmp, int statics)
{
    const Tile tile = tiles[blockIdx.x];
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    if (i >= tile.end) return;
    const float4 p = in[2 * (size_t)i];
    const float4 v = in[2 * (size_t)i + 1];
    const uint32_t w = statics ? cell_hash(p.x, p.y, p.z, sc.h) : i - sc.p_off;
    pos_tmp[i] = make_float4(p.x, p.y, p.z, __uint_as_float(w));
    vel_tmp[i] = make_float4(v.x, v.y, v.z, statics ? 0.f : p.w);
}

// The same load straight from the caller's arrays: positions (and
// velocities, or none) as 3 floats per particle in the caller's order,
// element k of the view at slot p_off + k.  Used where the GPU reads
// pageable host memory directly (Grace's address translation on GB300), so
// a job's particles need neither a host repack nor a staging copy.
__global__ void __launch_bounds__(kTileThreads) k_load_points(const Tile* tiles, const SceneDesc* scenes,
                                                              const float* p3, const float* v3, float4* pos_tmp,
                                                              float4* vel_tmp, int statics)
{
    const Tile tile = tiles[blockIdx.x];
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    if (i >= tile.end) return;
    const size_t k = i - sc.p_off;
    const float x = p3[3 * k], y = p3[3 * k + 1], z = p3[3 * k + 2];
    float vx = 0.f, vy = 0.f, vz = 0.f;
    if (v3) {
        vx = v3[3 * k];
        vy = v3[3 * k + 1];
        vz = v3[3 * k + 2];
    }
    const uint32_t w = statics ? cell_hash(x, y, z, sc.h) : (uint32_t)k;
    pos_tmp[i] = make_float4(x, y, z, __uint_as_float(w));
    vel_tmp[i] = make_float4(vx, vy, vz, 0.f);
}

// The tile table of a scene table, built on the device: tile t belongs to
// the scene k with first[k] <= t < first[k + 1] (first[n_scenes] = total)
// and covers kTileThreads slots of it.
__global__ void __launch_bounds__(kTileThreads) k_build_tiles(const SceneDesc* scenes, const uint32_t* first,
                                                              uint32_t n_scenes, Tile* out, uint32_t total)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    uint32_t lo = 0, hi = n_scenes;          // the last scene whose first tile is <= t
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (first[mid] <= t) lo = mid; else hi = mid;
    }
    const SceneDesc& d = scenes[lo];
    const uint32_t b = (t - first[lo]) * (uint32_t)kTileThreads;
    out[t] = Tile{lo, d.p_off + b, d.p_off + min(b + (uint32_t)kTileThreads, d.n), 0u};
}

// ---------------------------------------------------------------------------
// StepState host side
// ---------------------------------------------------------------------------

// Failure-detection probe: the scan kernel on two tiles of zeros, launched for
// tile 1 alone (the ticket starts at 1), so tile 1's look-back waits for a tile
// 0 that is never published.  The bounded wait expires, sets the status bit
// and lets the kernel finish; every access stays inside the probe's arrays.
sph_status scan_wait_probe(int device, uint32_t* status_bits)
{
    CUDA_TRY(cudaSetDevice(device));
    const uint32_t len = 2u * kScanTile;
    uint32_t *cnt = nullptr, *out = nullptr, *ticket = nullptr, *err = nullptr;
    unsigned long long* status = nullptr;
    sph_status st = SPH_OK;
    if ((st = dev_alloc(&cnt, len)) == SPH_OK && (st = dev_alloc(&out, len)) == SPH_OK &&
        (st = dev_alloc(&ticket, 1)) == SPH_OK && (st = dev_alloc(&err, 1)) == SPH_OK &&
        (st = dev_alloc(&status, 2)) == SPH_OK) {
        const uint32_t one = 1u;
        cudaError_t e = cudaMemset(cnt, 0, sizeof(uint32_t) * len);
        if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(unsigned long long) * 2);
        if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemcpy(ticket, &one, sizeof(uint32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            k_scan<<<1, kScanThreads>>>(cnt, out, len, status, ticket, err);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(status_bits, err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_last_error(std::string("wait probe: ") + cudaGetErrorString(e));
            st = SPH_ERR_CUDA;
        }
    }
    for (void* p : {(void*)cnt, (void*)out, (void*)ticket, (void*)err, (void*)status})
        if (p) cudaFree(p);
    if (st != SPH_OK) return st;
    if (*status_bits & DEV_ERR_SCAN_TIMEOUT) {
        set_last_error("device status 0x1 (scan wait expired)");
        return SPH_ERR_DEVICE_TIMEOUT;
    }
    return SPH_OK;
}

thread_local std::string g_last_error;

void set_last_error(const std::string& s) { g_last_error = s; }
const char* last_error() { return g_last_error.c_str(); }

StepState::~StepState() { release(); }

// Drops the scenes (host tables, the step graph, the triangle cells) and
// keeps every other device array for the next build.
void StepState::drop_scenes()
{
    drop_graphs();
    if (tri_cells) { cudaFree(tri_cells); tri_cells = nullptr; }
    if (tri_list) { cudaFree(tri_list); tri_list = nullptr; }
    scenes.clear();
    tiles.clear();
    stiles.clear();
    tile_first_.clear();
    total_n = total_s = total_t = 0;
    scan_len = sscan_len = sfscan_len = 0;
}

void StepState::release()
{
    drop_scenes();
    free_device_arrays();
}

void StepState::free_device_arrays()
{
    void* ptrs[] = {d_scenes, d_sscenes, d_sfscenes, d_tiles, d_stiles, pos, vel, pos_tmp, vel_tmp, key, arrival,
                    ptag, count, start, scan_status, scan_ticket, err, bar, nonfinite, spos, sstart, spos_ref,
                    sstart_ref, tris,
                    accel, accel_tmp, accel_io, staging, d_tmp_tiles_, d_tmp_scene_, nbr, snbr, ncount, tile_overflow,
                    saved_pos_, saved_vel_, saved_start_, sbitmap, tag, tag_io, rank_io, saved_tag_, tri_cells, tri_list,
                    render_zkey_, render_rgba_, render_depth_, d_tile_first_};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    d_scenes = d_sscenes = d_sfscenes = d_tmp_scene_ = nullptr;
    if (err_host_) { cudaFreeHost(err_host_); err_host_ = nullptr; }
    saved_pos_ = saved_vel_ = nullptr;
    saved_start_ = nullptr;
    tag = tag_io = rank_io = saved_tag_ = nullptr;
    tri_cells = tri_list = nullptr;
    render_zkey_ = nullptr;
    render_rgba_ = nullptr;
    render_depth_ = nullptr;
    render_pixels_ = 0;
    grid_cache_ = 0;
    spos_ref = nullptr;
    sstart_ref = nbr = snbr = ncount = tile_overflow = sbitmap = nullptr;
    d_tiles = d_stiles = d_tmp_tiles_ = nullptr;
    d_tile_first_ = nullptr;
    pos = vel = pos_tmp = vel_tmp = spos = accel = accel_tmp = accel_io = nullptr;
    staging = nullptr;
    key = arrival = ptag = count = start = scan_ticket = err = bar = nonfinite = sstart = nullptr;
    scan_status = nullptr;
    tris = nullptr;
    for (auto& e : events_)
        if (e) cudaEventDestroy(e);
    for (auto& e : events_) e = nullptr;
    cap_n_ = cap_q_ = cap_s_ = cap_sq_ = cap_sf_ = cap_sbm_ = cap_t_ = max_scenes_ = max_tiles_ = 0;
}

static SceneDesc make_scene_desc(const sph_params& p, float dt)
{
    SceneDesc d{};
    d.h = p.max_interaction_distance;
    d.h2 = d.h * d.h;
    d.mass = p.particle_mass;
    d.gas = p.gas_constant;
    d.rho0 = p.rest_density;
    d.visc = p.viscosity;
    d.gx = p.gravity_x;
    d.gy = p.gravity_y;
    d.gz = p.gravity_z;
    d.kc = kernel_constant(d.h);
    d.self_density = self_density(d.mass, d.h, d.kc);
    d.dt = dt;
    return d;
}

SceneDesc scene_desc_for(const SceneInput& in)
{
    SceneDesc d = make_scene_desc(in.params, in.dt);
    d.n = in.n;
    d.buckets = in.buckets ? in.buckets : 2u * in.n;
    d.s = in.s;
    d.t = in.t;
    d.fm_b = make_fastmod(d.buckets);
    d.fm_s = make_fastmod(in.s);
    d.sf_buckets = fast_static_buckets(in.s);
    d.fm_sf = make_fastmod(d.sf_buckets);
    d.sbm_mask = in.s ? static_bitmap_bits(in.s) - 1u : 0u;
    return d;
}

// ---- triangle cells ---------------------------------------------------------
//
// A uniform grid over the triangles' box grown by the reach; each cell lists,
// in increasing index, every triangle whose box grown by the reach (plus a
// margin for the rounding of the distance) reaches into the cell.  A point's
// cell is floor((p - o) * inv) in float, computed identically here and on the
// device; that is monotone in p, so every point within reach of a triangle
// lands in a cell that lists it.  Cells are half the reach wide, at most 96
// per axis; a grid that would list more than 2^26 entries is coarsened.
static float cell_of(float x, float o, float inv)
{
    volatile float d = x - o;   // rounded as on the device: no contraction
    volatile float m = d * inv;
    return std::floor((float)m);
}

static bool build_triangle_cells(const float* tris, uint32_t t, uint32_t t_off, SceneDesc& d,
                                 std::vector<uint32_t>& cells, std::vector<uint32_t>& list)
{
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float mag = 0.f;
    for (size_t k = 0; k < 9ull * t; ++k) {
        const float v = tris[k];
        if (!std::isfinite(v)) return false;   // no cells: every triangle for every particle
        lo[k % 3] = std::min(lo[k % 3], v);
        hi[k % 3] = std::max(hi[k % 3], v);
        mag = std::max(mag, std::fabs(v));
    }
    const float reach = kTriangleReach + 1e-4f * (kTriangleReach + mag) + 1e-6f;
    float o[3], ext = 0.f;
    for (int a = 0; a < 3; ++a) {
        o[a] = lo[a] - reach;
        ext = std::max(ext, (hi[a] + reach) - o[a]);
    }
    for (float cs = std::max(0.5f * kTriangleReach, ext / 96.f);; cs *= 1.5f) {
        const float inv = 1.0f / cs;
        uint32_t n[3];
        for (int a = 0; a < 3; ++a) n[a] = (uint32_t)cell_of(hi[a] + reach, o[a], inv) + 1u;
        const uint64_t ncell = (uint64_t)n[0] * n[1] * n[2];
        // per triangle: its cell range on each axis
        std::vector<uint32_t> r(6ull * t);
        uint64_t total = 0;
        for (uint32_t k = 0; k < t; ++k) {
            const float* v = tris + 9ull * k;
            uint64_t cnt = 1;
            for (int a = 0; a < 3; ++a) {
                const float tlo = std::min(std::min(v[a], v[3 + a]), v[6 + a]);
                const float thi = std::max(std::max(v[a], v[3 + a]), v[6 + a]);
                const float c0 = std::max(cell_of(tlo - reach, o[a], inv), 0.f);
                const float c1 = std::min(cell_of(thi + reach, o[a], inv), (float)(n[a] - 1));
                r[6ull * k + 2 * a] = (uint32_t)c0;
                r[6ull * k + 2 * a + 1] = (uint32_t)c1;
                cnt *= (uint64_t)(c1 - c0 + 1.f);
            }
            total += cnt;
        }
        if (total > (1ull << 26) && ncell > 1) continue;
        const uint32_t base = (uint32_t)cells.size();
        std::vector<uint32_t> count(ncell + 1, 0);
        auto each_cell = [&](uint32_t k, auto&& fn) {
            const uint32_t* q = &r[6ull * k];
            for (uint32_t z = q[4]; z <= q[5]; ++z)
                for (uint32_t y = q[2]; y <= q[3]; ++y)
                    for (uint32_t x = q[0]; x <= q[1]; ++x) fn(((uint64_t)z * n[1] + y) * n[0] + x);
        };
        for (uint32_t k = 0; k < t; ++k) each_cell(k, [&](uint64_t c) { ++count[c + 1]; });
        for (uint64_t c = 0; c < ncell; ++c) count[c + 1] += count[c];
        const uint32_t lbase = (uint32_t)list.size();
        list.resize(list.size() + total);
        std::vector<uint32_t> fill(count.begin(), count.end() - 1);
        for (uint32_t k = 0; k < t; ++k)   // increasing k: each cell's list stays in triangle order
            each_cell(k, [&](uint64_t c) { list[lbase + fill[c]++] = t_off + k; });
        for (uint64_t c = 0; c <= ncell; ++c) cells.push_back(lbase + count[c]);
        d.tg_ox = o[0];
        d.tg_oy = o[1];
        d.tg_oz = o[2];
        d.tg_inv = inv;
        d.tg_nx = n[0];
        d.tg_ny = n[1];
        d.tg_nz = n[2];
        d.tg_cell_off = base;
        return true;
    }
}

// The same scene with a static index space in the dynamic fields, so the
// sort kernels serve both particle kinds: the reference's s-bucket table
// (fast = false) or the neighbour-pass table (fast = true).
static SceneDesc static_view(SceneDesc d, bool fast)
{
    d.p_off = d.s_off;
    d.n = d.s;
    d.q_off = fast ? d.sf_off : d.sq_off;
    d.buckets = fast ? d.sf_buckets : d.s;
    d.fm_b = fast ? d.fm_sf : d.fm_s;
    return d;
}

sph_status validate_scene(const SceneInput& in)
{
    const sph_params& p = in.params;
    if (!(p.max_interaction_distance > 0.f) || !std::isfinite(p.max_interaction_distance)) {
        set_last_error("max_interaction_distance must be a positive finite number");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (!(p.gas_constant != 0.f)) {
        set_last_error("gas_constant must be non-zero (the force pass divides by it)");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (in.n && !in.pos) { set_last_error("dyn_pos is null"); return SPH_ERR_INVALID_ARGUMENT; }
    if (in.s && !in.spos) { set_last_error("static_pos is null"); return SPH_ERR_INVALID_ARGUMENT; }
    if (in.t && !in.tris) { set_last_error("triangles is null"); return SPH_ERR_INVALID_ARGUMENT; }
    if (in.n > kMaxParticles || in.s > kMaxParticles) {
        set_last_error("particle count exceeds 2^30");
        return SPH_ERR_CAPACITY;
    }
    return SPH_OK;
}

static uint32_t tiles_for(uint32_t n) { return (n + kTileThreads - 1) / kTileThreads; }

// Allocates every device array for the given capacities (all zero-filled
// where the algorithm needs zeros: bucket counters, scan status, errors).
sph_status StepState::alloc_arrays(uint32_t cap_n, uint32_t cap_q, uint32_t cap_s, uint32_t cap_sq, uint32_t cap_sf,
                                   uint32_t cap_sbm, uint32_t cap_t, uint32_t max_scenes, uint32_t max_tiles)
{
    cap_sbm_ = cap_sbm;
    cap_n_ = cap_n;
    cap_q_ = cap_q;
    cap_s_ = cap_s;
    cap_sq_ = cap_sq;
    cap_sf_ = cap_sf;
    cap_t_ = cap_t;
    max_scenes_ = std::max<uint32_t>(1, max_scenes);
    max_tiles_ = std::max<uint32_t>(1, max_tiles);
    const uint32_t work_n = std::max(cap_n, cap_s);
    const uint32_t cnt_len = std::max(std::max(cap_q, cap_sq), cap_sf) + 1u;
    const uint32_t scan_tiles_max = (cnt_len + kScanTile - 1) / kScanTile;
    sph_status st;
#define ALLOC(ptr, cnt) if ((st = dev_alloc(&(ptr), (cnt))) != SPH_OK) return st
    ALLOC(d_scenes, max_scenes_);
    ALLOC(d_sscenes, max_scenes_);
    ALLOC(d_sfscenes, max_scenes_);
    ALLOC(d_tiles, max_tiles_);
    ALLOC(d_stiles, max_tiles_);
    ALLOC(d_tmp_tiles_, tiles_for(work_n) + 1);
    ALLOC(d_tmp_scene_, 3);
    ALLOC(d_tile_first_, max_scenes_ + 1);
    ALLOC(pos, cap_n);
    ALLOC(vel, cap_n);
    ALLOC(pos_tmp, work_n);
    ALLOC(vel_tmp, work_n);
    ALLOC(key, work_n);
    ALLOC(arrival, work_n);
    ALLOC(ptag, work_n);
    ALLOC(tag, cap_n);
    ALLOC(tag_io, cap_n);
    ALLOC(count, cnt_len);
    ALLOC(start, cap_q + 1ull);
    ALLOC(scan_status, scan_tiles_max);
    ALLOC(scan_ticket, 1);
    ALLOC(err, 1);
    ALLOC(bar, 2);
    ALLOC(nonfinite, 2);
    ALLOC(spos, cap_s);
    ALLOC(sstart, cap_sf + 1ull);
    ALLOC(spos_ref, cap_s);
    ALLOC(sstart_ref, cap_sq + 1ull);
    ALLOC(nbr, (size_t)kMaxNbr * list_stride(cap_n));
    ALLOC(snbr, (size_t)kMaxSNbr * list_stride(cap_n));
    ALLOC(ncount, cap_n);
    ALLOC(tile_overflow, max_tiles_);
    ALLOC(sbitmap, cap_sbm);
    ALLOC(tris, 9ull * cap_t);
    ALLOC(staging, 2ull * work_n);
#undef ALLOC
    return zero_state_arrays();
}

// Zeroes the arrays the algorithm needs zero at the start of a build: bucket
// counters, scan status, status words, overflow flags, static bitmaps.
sph_status StepState::zero_state_arrays()
{
    const size_t cnt_len = std::max(std::max(cap_q_, cap_sq_), cap_sf_) + 1ull;
    const size_t scan_tiles_max = (cnt_len + kScanTile - 1) / kScanTile;
    CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(uint32_t) * cnt_len, stream_));
    CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), stream_));
    CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(uint32_t), stream_));
    CUDA_TRY(cudaMemsetAsync(nonfinite, 0, 2 * sizeof(uint32_t), stream_));
    CUDA_TRY(cudaMemsetAsync(scan_status, 0, sizeof(unsigned long long) * scan_tiles_max, stream_));
    CUDA_TRY(cudaMemsetAsync(tile_overflow, 0, sizeof(uint32_t) * max_tiles_, stream_));
    CUDA_TRY(cudaMemsetAsync(sbitmap, 0, sizeof(uint32_t) * std::max<uint32_t>(cap_sbm_, 1), stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

// Host positions (and velocities) of one scene -> staging as float4 pairs.
static sph_status upload_particles(cudaStream_t stream, float4* staging, uint32_t off, const float* p, const float* v,
                                   uint32_t n)
{
    if (!n) return SPH_OK;
    std::vector<float> hbuf(8ull * n, 0.f);
    for (uint32_t i = 0; i < n; ++i) {
        hbuf[8ull * i + 0] = p[3ull * i + 0];
        hbuf[8ull * i + 1] = p[3ull * i + 1];
        hbuf[8ull * i + 2] = p[3ull * i + 2];
        if (v) {
            hbuf[8ull * i + 4] = v[3ull * i + 0];
            hbuf[8ull * i + 5] = v[3ull * i + 1];
            hbuf[8ull * i + 6] = v[3ull * i + 2];
        }
    }
    // from pageable memory the call returns once the data is staged, so the
    // host buffer may be released right away; stream order does the rest
    CUDA_TRY(cudaMemcpyAsync(staging + 2ull * off, hbuf.data(), sizeof(float) * hbuf.size(), cudaMemcpyHostToDevice, stream));
    return SPH_OK;
}

sph_status StepState::build(int device, cudaStream_t stream, const std::vector<SceneInput>& inputs)
{
    drop_scenes();
    if (device != device_ || stream != stream_) free_device_arrays();
    device_ = device;
    stream_ = stream;
    uint64_t p_off = 0, q_off = 0, s_off = 0, sq_off = 0, sf_off = 0, sbm_off = 0, t_off = 0;
    for (size_t k = 0; k < inputs.size(); ++k) {
        const SceneInput& in = inputs[k];
        sph_status st = validate_scene(in);
        if (st != SPH_OK) return st;
        SceneDesc d = scene_desc_for(in);
        d.p_off = (uint32_t)p_off;
        d.q_off = (uint32_t)q_off;
        d.s_off = (uint32_t)s_off;
        d.sq_off = (uint32_t)sq_off;
        d.sf_off = (uint32_t)sf_off;
        d.sbm_off = (uint32_t)sbm_off;
        d.t_off = (uint32_t)t_off;
        scenes.push_back(d);
        tile_first_.push_back((uint32_t)tiles.size());
        for (uint32_t b = 0; b < in.n; b += kTileThreads)
            tiles.push_back(Tile{(uint32_t)k, (uint32_t)(p_off + b), (uint32_t)(p_off + std::min<uint64_t>(b + kTileThreads, in.n)), 0});
        for (uint32_t b = 0; b < in.s; b += kTileThreads)
            stiles.push_back(Tile{(uint32_t)k, (uint32_t)(s_off + b), (uint32_t)(s_off + std::min<uint64_t>(b + kTileThreads, in.s)), 0});
        p_off += in.n;
        q_off += d.buckets;
        s_off += in.s;
        sq_off += in.s;
        sf_off += d.sf_buckets;
        sbm_off += in.s ? (d.sbm_mask + 1ull) / 32 : 0;
        t_off += in.t;
        if (p_off > kMaxParticles || s_off > kMaxParticles || q_off >= (1ull << 31) || sf_off >= (1ull << 31)) {
            set_last_error("total particle or bucket count exceeds the 32-bit index space");
            return SPH_ERR_CAPACITY;
        }
    }
    total_n = (uint32_t)p_off;
    total_s = (uint32_t)s_off;
    total_t = (uint32_t)t_off;
    std::vector<uint32_t> tcells, tlist;
    for (size_t k = 0; k < inputs.size(); ++k)
        if (inputs[k].t) build_triangle_cells(inputs[k].tris, inputs[k].t, scenes[k].t_off, scenes[k], tcells, tlist);
    scan_len = (uint32_t)q_off + 1u;
    sscan_len = (uint32_t)sq_off + 1u;
    sfscan_len = (uint32_t)sf_off + 1u;
    // the arrays of an earlier build are reused when every capacity fits
    const size_t need_tiles = std::max(tiles.size(), stiles.size());
    const bool fits = pos && total_n <= cap_n_ && q_off <= cap_q_ && total_s <= cap_s_ && sq_off <= cap_sq_ &&
                      sf_off <= cap_sf_ && sbm_off <= cap_sbm_ && total_t <= cap_t_ &&
                      scenes.size() <= max_scenes_ && need_tiles <= max_tiles_;
    sph_status st;
    if (fits) {
        st = zero_state_arrays();
    } else {
        free_device_arrays();
        st = alloc_arrays(total_n, (uint32_t)q_off, total_s, (uint32_t)sq_off, (uint32_t)sf_off, (uint32_t)sbm_off,
                          total_t, (uint32_t)scenes.size(), (uint32_t)need_tiles);
    }
    if (st != SPH_OK) return st;
    if (!tcells.empty()) {
        if ((st = dev_alloc(&tri_cells, tcells.size())) != SPH_OK) return st;
        if ((st = dev_alloc(&tri_list, std::max<size_t>(tlist.size(), 1))) != SPH_OK) return st;
        CUDA_TRY(cudaMemcpyAsync(tri_cells, tcells.data(), sizeof(uint32_t) * tcells.size(), cudaMemcpyHostToDevice, stream_));
        if (!tlist.empty())
            CUDA_TRY(cudaMemcpyAsync(tri_list, tlist.data(), sizeof(uint32_t) * tlist.size(), cudaMemcpyHostToDevice, stream_));
    }
    std::vector<SceneDesc> sview, sfview;
    for (const auto& d : scenes) {
        sview.push_back(static_view(d, false));
        sfview.push_back(static_view(d, true));
    }
    CUDA_TRY(cudaMemcpyAsync(d_sfscenes, sfview.data(), sizeof(SceneDesc) * sfview.size(), cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(d_scenes, scenes.data(), sizeof(SceneDesc) * scenes.size(), cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(d_sscenes, sview.data(), sizeof(SceneDesc) * sview.size(), cudaMemcpyHostToDevice, stream_));
    if (!tiles.empty())
        CUDA_TRY(cudaMemcpyAsync(d_tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, stream_));
    if (!stiles.empty())
        CUDA_TRY(cudaMemcpyAsync(d_stiles, stiles.data(), sizeof(Tile) * stiles.size(), cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));

    // statics of every scene first (staging is their scratch), then dynamics
    for (size_t k = 0; k < inputs.size(); ++k) {
        if ((st = upload_particles(stream_, staging, scenes[k].s_off, inputs[k].spos, nullptr, inputs[k].s)) != SPH_OK)
            return st;
        if (inputs[k].t)
            CUDA_TRY(cudaMemcpyAsync(tris + 9ull * scenes[k].t_off, inputs[k].tris, sizeof(float) * 9ull * inputs[k].t,
                                     cudaMemcpyHostToDevice, stream_));
    }
    if (total_s) {
        if ((st = enqueue_load(staging, /*statics=*/true)) != SPH_OK) return st;
        if ((st = enqueue_sort(1)) != SPH_OK) return st;
        if ((st = enqueue_sort(2)) != SPH_OK) return st;
        k_static_bitmap<<<(unsigned)stiles.size(), kTileThreads, 0, stream_>>>(d_stiles, d_scenes, spos, sbitmap);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(stream_));
    }
    for (size_t k = 0; k < inputs.size(); ++k)
        if ((st = upload_particles(stream_, staging, scenes[k].p_off, inputs[k].pos, inputs[k].vel, inputs[k].n)) != SPH_OK)
            return st;
    if (total_n) {
        if ((st = enqueue_load(staging, false)) != SPH_OK) return st;
        if ((st = enqueue_sort(0)) != SPH_OK) return st;
    }
    return check_device_error();
}

// ---- arena mode ---------------------------------------------------------------

sph_status StepState::init_arena(int device, cudaStream_t stream, uint32_t cap_n, uint32_t cap_q, uint32_t cap_s,
                                 uint32_t cap_sq, uint32_t cap_sf, uint32_t cap_sbm, uint32_t max_scenes)
{
    release();
    device_ = device;
    stream_ = stream;
    return alloc_arrays(cap_n, cap_q, cap_s, cap_sq, cap_sf, cap_sbm, 0, max_scenes, tiles_for(cap_n) + max_scenes);
}

template <typename T>
static sph_status grow_one(T** p, size_t old_count, size_t new_count, bool zero_tail, cudaStream_t stream)
{
    T* q = nullptr;
    sph_status st = dev_alloc(&q, new_count);
    if (st != SPH_OK) return st;
    if (*p && old_count)
        CUDA_TRY(cudaMemcpyAsync(q, *p, sizeof(T) * old_count, cudaMemcpyDeviceToDevice, stream));
    if (zero_tail && new_count > old_count)
        CUDA_TRY(cudaMemsetAsync(q + old_count, 0, sizeof(T) * (new_count - old_count), stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (*p) cudaFree(*p);
    *p = q;
    return SPH_OK;
}

sph_status StepState::grow_arena(uint32_t cap_n, uint32_t cap_q, uint32_t cap_s, uint32_t cap_sq, uint32_t cap_sf,
                                 uint32_t cap_sbm)
{
    cap_n = std::max(cap_n, cap_n_);
    cap_q = std::max(cap_q, cap_q_);
    cap_s = std::max(cap_s, cap_s_);
    cap_sq = std::max(cap_sq, cap_sq_);
    cap_sf = std::max(cap_sf, cap_sf_);
    cap_sbm = std::max(cap_sbm, cap_sbm_);
    if (cap_n == cap_n_ && cap_q == cap_q_ && cap_s == cap_s_ && cap_sq == cap_sq_ && cap_sf == cap_sf_ &&
        cap_sbm == cap_sbm_)
        return SPH_OK;
    drop_graphs();
    const size_t old_work = std::max(cap_n_, cap_s_), new_work = std::max(cap_n, cap_s);
    const size_t old_cnt = std::max(std::max(cap_q_, cap_sq_), cap_sf_) + 1ull;
    const size_t new_cnt = std::max(std::max(cap_q, cap_sq), cap_sf) + 1ull;
    const size_t new_scan_tiles = (new_cnt + kScanTile - 1) / kScanTile;
    sph_status st;
#define GROW(ptr, o, nw, z) if ((st = grow_one(&(ptr), (o), (nw), (z), stream_)) != SPH_OK) return st
    GROW(pos, cap_n_, cap_n, false);
    GROW(vel, cap_n_, cap_n, false);
    GROW(pos_tmp, old_work, new_work, false);
    GROW(vel_tmp, old_work, new_work, false);
    GROW(key, old_work, new_work, false);
    GROW(arrival, old_work, new_work, false);
    GROW(ptag, old_work, new_work, false);
    GROW(tag, cap_n_, cap_n, false);
    GROW(tag_io, 0, cap_n, false);
    GROW(staging, 2 * old_work, 2 * new_work, false);
    GROW(count, old_cnt, new_cnt, true);
    GROW(start, cap_q_ + 1ull, cap_q + 1ull, false);
    GROW(spos, cap_s_, cap_s, false);
    GROW(sstart, cap_sf_ + 1ull, cap_sf + 1ull, false);
    GROW(spos_ref, cap_s_, cap_s, false);
    GROW(sstart_ref, cap_sq_ + 1ull, cap_sq + 1ull, false);
    GROW(nbr, 0, (size_t)kMaxNbr * list_stride(cap_n), false);
    GROW(snbr, 0, (size_t)kMaxSNbr * list_stride(cap_n), false);
    GROW(ncount, 0, cap_n, false);
    GROW(tile_overflow, 0, tiles_for(cap_n) + max_scenes_, true);
    GROW(sbitmap, cap_sbm_, std::max<uint32_t>(cap_sbm, 1), true);
    GROW(scan_status, 0, new_scan_tiles, true);
    GROW(d_tmp_tiles_, 0, tiles_for((uint32_t)new_work) + 1, false);
    GROW(d_tiles, 0, tiles_for(cap_n) + max_scenes_, false);
    GROW(d_stiles, 0, tiles_for(cap_n) + max_scenes_, false);
#undef GROW
    if (accel) { cudaFree(accel); accel = nullptr; }
    if (accel_tmp) { cudaFree(accel_tmp); accel_tmp = nullptr; }
    if (accel_io) { cudaFree(accel_io); accel_io = nullptr; }
    if (rank_io) { cudaFree(rank_io); rank_io = nullptr; }
    max_tiles_ = tiles_for(cap_n) + max_scenes_;
    cap_n_ = cap_n;
    cap_q_ = cap_q;
    cap_s_ = cap_s;
    cap_sq_ = cap_sq;
    cap_sf_ = cap_sf;
    cap_sbm_ = cap_sbm;
    return set_active(scenes);
}

// Sorts one scene alone: its own tiles and one-entry scene tables, and scans
// over its own bucket ranges only, so every other scene's table is untouched
// (a sub-range scan yields local starts; the per-scene delta absorbs that).
sph_status StepState::admit_scene(const SceneDesc& d, const SceneInput& in, bool sync, bool host_direct)
{
    if (d.p_off + (uint64_t)d.n > cap_n_ || d.q_off + (uint64_t)d.buckets > cap_q_ ||
        d.s_off + (uint64_t)d.s > cap_s_ || d.sq_off + (uint64_t)d.s > cap_sq_ ||
        d.sf_off + (uint64_t)d.sf_buckets > cap_sf_ || (d.s && d.sbm_off + (d.sbm_mask + 1ull) / 32 > cap_sbm_)) {
        set_last_error("scene ranges exceed the arena");
        return SPH_ERR_CAPACITY;
    }
    if ((d.q_off & 3u) || (d.sq_off & 3u) || (d.sf_off & 3u)) {
        set_last_error("bucket ranges must start on a multiple of 4");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    // views: 0 dynamic, 1 statics by the reference's table, 2 by the
    // neighbour-pass table
    SceneDesc views[3] = {d, static_view(d, false), static_view(d, true)};
    CUDA_TRY(cudaMemcpyAsync(d_tmp_scene_, views, sizeof(views), cudaMemcpyHostToDevice, stream_));
    std::vector<Tile> tl;
    sph_status st;
    for (int kind : {1, 2, 0}) {
        const SceneDesc& v = views[kind];
        if (!v.n) continue;
        tl.clear();
        for (uint32_t b = 0; b < v.n; b += kTileThreads)
            tl.push_back(Tile{(uint32_t)kind, v.p_off + b, v.p_off + std::min<uint32_t>(b + kTileThreads, v.n), 0});
        CUDA_TRY(cudaMemcpyAsync(d_tmp_tiles_, tl.data(), sizeof(Tile) * tl.size(), cudaMemcpyHostToDevice, stream_));
        const unsigned nt = (unsigned)tl.size();
        if (kind != 2) {   // the second static sort reuses the first one's loaded particles
            if (host_direct) {
                k_load_points<<<nt, kTileThreads, 0, stream_>>>(d_tmp_tiles_, d_tmp_scene_,
                                                                kind == 1 ? in.spos : in.pos,
                                                                kind == 1 ? nullptr : in.vel, pos_tmp, vel_tmp,
                                                                kind != 0 ? 1 : 0);
            } else {
                if (kind == 1) {
                    if ((st = upload_particles(stream_, staging, v.p_off, in.spos, nullptr, v.n)) != SPH_OK) return st;
                } else {
                    if ((st = upload_particles(stream_, staging, v.p_off, in.pos, in.vel, v.n)) != SPH_OK) return st;
                }
                k_load<<<nt, kTileThreads, 0, stream_>>>(d_tmp_tiles_, d_tmp_scene_, staging, pos_tmp, vel_tmp,
                                                         kind != 0 ? 1 : 0);
            }
            CUDA_TRY(cudaGetLastError());
        }
        SortArgs a = sort_args(kind);
        a.tiles = d_tmp_tiles_;
        a.scenes = d_tmp_scene_;
        k_hash_count<<<nt, kTileThreads, 0, stream_>>>(a);
        CUDA_TRY(cudaGetLastError());
        if ((st = enqueue_scan(count + v.q_off, a.start + v.q_off, v.buckets + 1u)) != SPH_OK) return st;
        k_scatter<<<nt, kTileThreads, 0, stream_>>>(a);
        CUDA_TRY(cudaGetLastError());
        k_gather<<<nt, kTileThreads, 0, stream_>>>(a);
        CUDA_TRY(cudaGetLastError());
        if (kind == 2) {   // this scene's static-presence bitmap, from its sorted statics
            CUDA_TRY(cudaMemsetAsync(sbitmap + d.sbm_off, 0, sizeof(uint32_t) * ((d.sbm_mask + 1ull) / 32), stream_));
            k_static_bitmap<<<nt, kTileThreads, 0, stream_>>>(d_tmp_tiles_, d_tmp_scene_, spos, sbitmap);
            CUDA_TRY(cudaGetLastError());
        }
    }
    return sync ? check_device_error() : SPH_OK;
}

sph_status StepState::set_active(const std::vector<SceneDesc>& descs)
{
    if (descs.size() > max_scenes_) {
        set_last_error("more scenes than the arena's slots");
        return SPH_ERR_CAPACITY;
    }
    drop_graphs();
    scenes = descs;
    tile_first_.clear();
    uint64_t qmax = 0, tn = 0, nt = 0;
    for (size_t k = 0; k < scenes.size(); ++k) {
        const SceneDesc& d = scenes[k];
        tile_first_.push_back((uint32_t)nt);
        nt += (d.n + kTileThreads - 1) / kTileThreads;
        qmax = std::max<uint64_t>(qmax, (uint64_t)d.q_off + d.buckets);
        tn += d.n;
    }
    if (nt > max_tiles_) {
        set_last_error("tile table overflow");
        return SPH_ERR_CAPACITY;
    }
    // the host keeps only the count; the table itself is built on the device
    tiles.resize(nt);
    total_n = (uint32_t)tn;
    scan_len = (uint32_t)qmax + 1u;
    if (!scenes.empty()) {
        std::vector<uint32_t> first(tile_first_);
        first.push_back((uint32_t)nt);
        // copies from pageable memory are staged when the call returns, so
        // the host tables may change right away; stream order does the rest
        CUDA_TRY(cudaMemcpyAsync(d_scenes, scenes.data(), sizeof(SceneDesc) * scenes.size(), cudaMemcpyHostToDevice, stream_));
        CUDA_TRY(cudaMemcpyAsync(d_tile_first_, first.data(), sizeof(uint32_t) * first.size(), cudaMemcpyHostToDevice,
                                 stream_));
        if (nt) {
            k_build_tiles<<<(unsigned)((nt + kTileThreads - 1) / kTileThreads), kTileThreads, 0, stream_>>>(
                d_scenes, d_tile_first_, (uint32_t)scenes.size(), d_tiles, (uint32_t)nt);
            CUDA_TRY(cudaGetLastError());
        }
    }
    return SPH_OK;
}

// ---- launches -------------------------------------------------------------------

sph_status StepState::enqueue_load(const float4* src, bool statics)
{
    const std::vector<Tile>& tl = statics ? stiles : tiles;
    if (tl.empty()) return SPH_OK;
    k_load<<<(unsigned)tl.size(), kTileThreads, 0, stream_>>>(statics ? d_stiles : d_tiles, statics ? d_sscenes : d_scenes,
                                                                src, pos_tmp, vel_tmp, statics ? 1 : 0);
    CUDA_TRY(cudaGetLastError());
    return SPH_OK;
}

// The sorts outside a step: kind 0 loads dynamic particles (the initial
// sort numbers their tags by slot, like the reference's initial reorder,
// SimulationEngineCPU.cpp:69-128), kinds 1 and 2 statics (no tags).
SortArgs StepState::sort_args(int kind) const
{
    SortArgs a{};
    a.tiles = kind == 0 ? d_tiles : d_stiles;
    a.scenes = kind == 0 ? d_scenes : (kind == 1 ? d_sscenes : d_sfscenes);
    a.pos_src = pos_tmp;
    a.vel_src = vel_tmp;
    a.pos_dst = kind == 0 ? pos : (kind == 1 ? spos_ref : spos);
    a.vel_dst = kind == 0 ? vel : staging;   // static velocities are discarded
    a.key = key;
    a.arrival = arrival;
    a.ptag = ptag;
    a.tag_src = nullptr;
    a.tag_dst = kind == 0 ? tag : nullptr;
    a.assign = kind == 0 ? kTagSlot : kTagNone;
    a.count = count;
    a.start = kind == 0 ? start : (kind == 1 ? sstart_ref : sstart);
    a.err = err;
    a.nonfinite_set = kind == 0 ? nonfinite : nullptr;   // dynamic sorts mark the current word
    a.nonfinite_rotate = nullptr;
    return a;
}

// Counting sort of the tmp arrays into a sorted array: hash + count, scan,
// scatter, stable gather (positions must already be in pos_tmp, and stay
// there, so both static sorts read the same load).
sph_status StepState::enqueue_sort(int kind, bool keep_tags)
{
    const std::vector<Tile>& tl = kind == 0 ? tiles : stiles;
    if (tl.empty()) return SPH_OK;
    SortArgs a = sort_args(kind);
    if (keep_tags) {   // a write between steps: rank by the slot before it, keep the tag
        a.tag_src = rank_io;
        a.tag_keep = tag_io;
        a.assign = kTagKeep;
    }
    const uint32_t len = kind == 0 ? scan_len : (kind == 1 ? sscan_len : sfscan_len);
    const unsigned nt = (unsigned)tl.size();
    k_hash_count<<<nt, kTileThreads, 0, stream_>>>(a);
    CUDA_TRY(cudaGetLastError());
    sph_status st = enqueue_scan(count, a.start, len);
    if (st != SPH_OK) return st;
    k_scatter<<<nt, kTileThreads, 0, stream_>>>(a);
    CUDA_TRY(cudaGetLastError());
    k_gather<<<nt, kTileThreads, 0, stream_>>>(a);
    CUDA_TRY(cudaGetLastError());
    return SPH_OK;
}

sph_status StepState::enqueue_scan(uint32_t* cnt, uint32_t* out, uint32_t len, bool cleared)
{
    const uint32_t tiles_n = (len + kScanTile - 1) / kScanTile;
    if (!cleared) {   // the step's overflow-force kernel clears them otherwise
        CUDA_TRY(cudaMemsetAsync(scan_status, 0, sizeof(unsigned long long) * tiles_n, stream_));
        CUDA_TRY(cudaMemsetAsync(scan_ticket, 0, sizeof(uint32_t), stream_));
    }
    k_scan<<<tiles_n, kScanThreads, 0, stream_>>>(cnt, out, len, scan_status, scan_ticket, err);
    CUDA_TRY(cudaGetLastError());
    return SPH_OK;
}

StepArgs StepState::step_args() const
{
    StepArgs a{};
    a.tiles = d_tiles;
    a.num_tiles = (uint32_t)tiles.size();
    a.scenes = d_scenes;
    a.pos = pos;
    a.vel = vel;
    a.pos_tmp = pos_tmp;
    a.vel_tmp = vel_tmp;
    a.key = key;
    a.arrival = arrival;
    a.ptag = ptag;
    a.tag = tag;
    a.count = count;
    a.start = start;
    a.scan_len = scan_len;
    a.scan_status = scan_status;
    a.scan_ticket = scan_ticket;
    a.spos = spos;
    a.sstart = sstart;
    a.spos_ref = spos_ref;
    a.sstart_ref = sstart_ref;
    a.tris = tris;
    a.tri_cells = tri_cells;
    a.tri_list = tri_list;
    a.sbitmap = sbitmap;
    a.accel = accel_tmp;
    a.err = err;
    a.nonfinite = nonfinite;
    a.bar_count = bar;
    a.bar_gen = bar + 1;
    a.nbr = nbr;
    a.snbr = snbr;
    a.ncount = ncount;
    a.tile_overflow = tile_overflow;
    a.nbr_stride = list_stride(cap_n_);
    return a;
}

sph_status StepState::ensure_events()
{
    for (auto& e : events_)
        if (!e) CUDA_TRY(cudaEventCreate(&e));
    return SPH_OK;
}

// One step as six launches (the overflow-force kernel clears the scan's
// look-back state, so no memset).  With `timed`, events bracket each stage
// on the launching stream.
template <bool kExact>
sph_status StepState::launch_step_staged(bool record_accel, bool timed)
{
    const unsigned nt = (unsigned)tiles.size();
    StepArgs a = step_args();
    SortArgs s = sort_args(0);
    s.tag_src = tag;          // the step's sort: tags per scene reorder flag
    s.tag_dst = tag;
    s.assign = kTagStep;
    s.nonfinite_set = nullptr;       // keys come from the force pass
    s.nonfinite_rotate = nonfinite;
    if (record_accel) {       // the recorded acceleration follows its particle
        s.accel_src = accel_tmp;
        s.accel_dst = accel;
    }
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(events_[0], stream_, cudaEventRecordExternal));
    if (!kExact && density_shape_ > 0)
        CUDA_TRY(launch_shaped(density_shape_, true, a, stream_));
    else
        k_density<kExact><<<nt, kDensityThreads, 0, stream_>>>(a);
    CUDA_TRY(cudaGetLastError());
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(events_[1], stream_, cudaEventRecordExternal));
    if (record_accel) {
        k_force<true, kExact><<<nt, kTileThreads, 0, stream_>>>(a);
        k_force_overflow<true, kExact><<<overflow_grid(nt), kTileThreads, 0, stream_>>>(a);
    } else {
        if (!kExact && force_shape_ > 0)
            CUDA_TRY(launch_shaped(force_shape_, false, a, stream_));
        else
            k_force<false, kExact><<<nt, kTileThreads, 0, stream_>>>(a);
        k_force_overflow<false, kExact><<<overflow_grid(nt), kTileThreads, 0, stream_>>>(a);
    }
    CUDA_TRY(cudaGetLastError());
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(events_[2], stream_, cudaEventRecordExternal));
    sph_status st = enqueue_scan(count, start, scan_len, /*cleared=*/true);
    if (st != SPH_OK) return st;
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(events_[3], stream_, cudaEventRecordExternal));
    k_scatter<<<nt, kTileThreads, 0, stream_>>>(s);
    CUDA_TRY(cudaGetLastError());
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(events_[4], stream_, cudaEventRecordExternal));
    k_gather<<<nt, kTileThreads, 0, stream_>>>(s);
    CUDA_TRY(cudaGetLastError());
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(events_[5], stream_, cudaEventRecordExternal));
    return SPH_OK;
}

// Grid of the overflow force pass: four CTAs per SM, at most one per tile.
unsigned StepState::overflow_grid(unsigned tiles_n)
{
    if (!sm_count_) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_) != cudaSuccess || sms < 1) sms = 1;
        sm_count_ = (uint32_t)sms;
    }
    return std::max(1u, std::min(tiles_n, 4u * sm_count_));
}

sph_status StepState::enqueue_step_staged(bool record_accel, bool timed)
{
    if (tiles.empty()) return SPH_OK;
    return exact_ ? launch_step_staged<true>(record_accel, timed) : launch_step_staged<false>(record_accel, timed);
}

static const void* persistent_kernel(bool exact)
{
    return exact ? (const void*)k_step_persistent<true> : (const void*)k_step_persistent<false>;
}

sph_status StepState::persistent_grid(uint32_t* grid)
{
    if (grid_cache_) {
        *grid = grid_cache_;
        return SPH_OK;
    }
    int sms = 0, per_sm = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_kernel(exact_), kTileThreads, 0));
    if (per_sm < 1) per_sm = 1;
    uint32_t g = (uint32_t)(sms * per_sm);
    if (persistent_ctas_ && persistent_ctas_ < g) g = persistent_ctas_;
    *grid = std::max<uint32_t>(1, g);
    grid_cache_ = *grid;
    return SPH_OK;
}

sph_status StepState::enqueue_step_persistent()
{
    if (tiles.empty()) return SPH_OK;
    uint32_t grid = 0;
    sph_status st = persistent_grid(&grid);
    if (st != SPH_OK) return st;
    StepArgs a = step_args();
    uint32_t scan_tiles = (scan_len + kScanTile - 1) / kScanTile;
    void* args[] = {&a, &scan_tiles};
    CUDA_TRY(cudaLaunchCooperativeKernel(persistent_kernel(exact_), dim3(grid), dim3(kTileThreads), args, 0, stream_));
    return SPH_OK;
}

// Captures one staged step into a graph (once per layout) and replays it.
sph_status StepState::enqueue_steps(uint32_t steps, StepMode mode, bool record_accel, bool timed)
{
    if (tiles.empty() || steps == 0) return SPH_OK;
    if (record_accel && !accel) {
        sph_status st = dev_alloc(&accel, total_n);
        if (st != SPH_OK) return st;
        st = dev_alloc(&accel_tmp, total_n);
        if (st != SPH_OK) return st;
        drop_graphs();
    }
    if (timed) {
        sph_status st = ensure_events();
        if (st != SPH_OK) return st;
        for (float& t : stage_ms_) t = 0.f;
        // the staged step is timed as it runs untimed: one graph launch per
        // step, here with event-record nodes between the stages
        const bool graphed = mode != StepMode::Persistent && !record_accel;
        if (graphed && !graph_timed_) {
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            st = enqueue_step_staged(false, true);
            cudaError_t e = cudaStreamEndCapture(stream_, &g);
            if (st != SPH_OK) { if (g) cudaGraphDestroy(g); return st; }
            if (e != cudaSuccess) { set_last_error(std::string("graph capture: ") + cudaGetErrorString(e)); return SPH_ERR_CUDA; }
            e = cudaGraphInstantiate(&graph_timed_, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                graph_timed_ = nullptr;
                set_last_error(std::string("graph instantiate: ") + cudaGetErrorString(e));
                return SPH_ERR_CUDA;
            }
        }
        for (uint32_t k = 0; k < steps; ++k) {
            if (graphed)
                CUDA_TRY(cudaGraphLaunch(graph_timed_, stream_));
            else
                st = (mode == StepMode::Persistent) ? enqueue_step_persistent() : enqueue_step_staged(record_accel, true);
            if (st != SPH_OK) return st;
            if (mode != StepMode::Persistent) {
                CUDA_TRY(cudaEventSynchronize(events_[5]));
                for (int s = 0; s < 5; ++s) {
                    float ms = 0.f;
                    CUDA_TRY(cudaEventElapsedTime(&ms, events_[s], events_[s + 1]));
                    stage_ms_[s] += ms;
                }
            }
        }
        return SPH_OK;
    }
    if (mode == StepMode::Persistent) {
        for (uint32_t k = 0; k < steps; ++k) {
            sph_status st = enqueue_step_persistent();
            if (st != SPH_OK) return st;
        }
        return SPH_OK;
    }
    if (record_accel) {
        for (uint32_t k = 0; k < steps; ++k) {
            sph_status st = enqueue_step_staged(true, false);
            if (st != SPH_OK) return st;
        }
        return SPH_OK;
    }
    if (!graph_) {
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        sph_status st = enqueue_step_staged(false, false);
        cudaError_t e = cudaStreamEndCapture(stream_, &g);
        if (st != SPH_OK) { if (g) cudaGraphDestroy(g); return st; }
        if (e != cudaSuccess) { set_last_error(std::string("graph capture: ") + cudaGetErrorString(e)); return SPH_ERR_CUDA; }
        e = cudaGraphInstantiate(&graph_, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { graph_ = nullptr; set_last_error(std::string("graph instantiate: ") + cudaGetErrorString(e)); return SPH_ERR_CUDA; }
    }
    for (uint32_t k = 0; k < steps; ++k) CUDA_TRY(cudaGraphLaunch(graph_, stream_));
    return SPH_OK;
}

// Waits for the stream and reads the device status word with one round trip:
// the word is copied into pinned host memory behind the queued work.
sph_status StepState::check_device_error()
{
    if (!err) {
        CUDA_TRY(cudaStreamSynchronize(stream_));
        return SPH_OK;
    }
    if (!err_host_) CUDA_TRY(cudaMallocHost((void**)&err_host_, sizeof(uint32_t)));
    CUDA_TRY(cudaMemcpyAsync(err_host_, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    const uint32_t h = *err_host_;
    if (h) {
        CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), stream_));
        CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(uint32_t), stream_));
        char msg[160];
        snprintf(msg, sizeof msg, "device status 0x%x (1 scan wait, 2 barrier wait, 4 slot range, 8 bucket range)", h);
        set_last_error(msg);
        return (h & (DEV_ERR_SCAN_TIMEOUT | DEV_ERR_BARRIER_TIMEOUT)) ? SPH_ERR_DEVICE_TIMEOUT : SPH_ERR_CUDA;
    }
    return SPH_OK;
}

sph_status StepState::set_dt(uint32_t scene, float dt)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    if (scenes[scene].dt == dt) return SPH_OK;
    scenes[scene].dt = dt;
    CUDA_TRY(cudaMemcpyAsync(&d_scenes[scene].dt, &scenes[scene].dt, sizeof(float), cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

sph_status StepState::set_reorder(uint32_t scene, bool reorder)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    const uint32_t r = reorder ? 1u : 0u;
    if (scenes[scene].reorder == r) return SPH_OK;
    scenes[scene].reorder = r;
    CUDA_TRY(cudaMemcpyAsync(&d_scenes[scene].reorder, &scenes[scene].reorder, sizeof(uint32_t), cudaMemcpyHostToDevice,
                             stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

// Reads one scene's particles (caller's order) into host `out` (n x 32 B).
sph_status StepState::read_scene(uint32_t scene, sph_dynamic_particle* out, float* accel_out, bool buffer_order)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    const SceneDesc& d = scenes[scene];
    if (!d.n) return SPH_OK;
    if (accel_out && !accel) { set_last_error("acceleration recording is off"); return SPH_ERR_INVALID_ARGUMENT; }
    if (accel_out && !accel_io) {
        sph_status st = dev_alloc(&accel_io, total_n);
        if (st != SPH_OK) return st;
    }
    const uint32_t t0 = tile_first_[scene];
    const uint32_t t1 = scene + 1 < tile_first_.size() ? tile_first_[scene + 1] : (uint32_t)tiles.size();
    if (t1 > t0)
        k_unsort<<<t1 - t0, kTileThreads, 0, stream_>>>(d_tiles + t0, d_scenes, pos, vel, staging,
                                                        accel_out ? accel : nullptr, accel_io, tag, nullptr,
                                                        buffer_order ? 1 : 0);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, staging + 2ull * d.p_off, sizeof(sph_dynamic_particle) * d.n, cudaMemcpyDeviceToHost, stream_));
    if (accel_out) {
        std::vector<float4> tmp(d.n);
        CUDA_TRY(cudaMemcpyAsync(tmp.data(), accel_io + d.p_off, sizeof(float4) * d.n, cudaMemcpyDeviceToHost, stream_));
        CUDA_TRY(cudaStreamSynchronize(stream_));
        for (uint32_t i = 0; i < d.n; ++i) {
            accel_out[3ull * i + 0] = tmp[i].x;
            accel_out[3ull * i + 1] = tmp[i].y;
            accel_out[3ull * i + 2] = tmp[i].z;
        }
    }
    return check_device_error();
}

// Queues the readback of one scene in the caller's order straight into host
// memory the GPU can write (pageable memory on a GPU with pageable memory
// access): no staging copy, no wait.  `out` must stay valid until the work
// completes.
sph_status StepState::read_scene_async(uint32_t scene, sph_dynamic_particle* out)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    const SceneDesc& d = scenes[scene];
    if (!d.n) return SPH_OK;
    const uint32_t t0 = tile_first_[scene];
    const uint32_t t1 = scene + 1 < tile_first_.size() ? tile_first_[scene + 1] : (uint32_t)tiles.size();
    if (t1 > t0)
        k_unsort<<<t1 - t0, kTileThreads, 0, stream_>>>(d_tiles + t0, d_scenes, pos, vel, reinterpret_cast<float4*>(out),
                                                        nullptr, nullptr, tag, nullptr, 0, nullptr, d.p_off);
    CUDA_TRY(cudaGetLastError());
    return SPH_OK;
}

// Replaces one scene's particles from host (caller's order) and re-sorts the
// whole state (other scenes are re-sorted unchanged).
sph_status StepState::write_scene(uint32_t scene, const sph_dynamic_particle* in, bool wait)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    const SceneDesc& d = scenes[scene];
    if (!d.n) return SPH_OK;
    // move the current sorted state of all scenes, their buffer tags and their
    // slots into staging order first (a lone scene is replaced whole: its tags
    // and slots only).  The re-sort keeps every particle's tag, and inside a
    // bucket keeps the order the particles had: the reference's LockWrite
    // changes the buffer, not its maps, so a written-back state must visit its
    // neighbours as before (after a reordering step that order is by rising
    // tag, after a map-mode step by falling tag).
    if (!rank_io) {
        sph_status st = dev_alloc(&rank_io, cap_n_);
        if (st != SPH_OK) return st;
    }
    k_unsort<<<(unsigned)tiles.size(), kTileThreads, 0, stream_>>>(d_tiles, d_scenes, pos, vel,
                                                                   scenes.size() > 1 ? staging : nullptr, nullptr,
                                                                   nullptr, tag, tag_io, 0, rank_io);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(staging + 2ull * d.p_off, in, sizeof(sph_dynamic_particle) * d.n, cudaMemcpyHostToDevice, stream_));
    sph_status st = enqueue_load(staging, false);
    if (st != SPH_OK) return st;
    // the re-sort hashes every particle again: it recomputes the flag
    CUDA_TRY(cudaMemsetAsync(nonfinite, 0, 2 * sizeof(uint32_t), stream_));
    st = enqueue_sort(0, /*keep_tags=*/true);
    if (st != SPH_OK) return st;
    return wait ? check_device_error() : SPH_OK;
}

sph_status StepState::read_static(uint32_t scene, sph_static_particle* out, uint32_t* bucket_starts)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    const SceneDesc& d = scenes[scene];
    if (!d.s) return SPH_OK;
    if (out) {
        CUDA_TRY(cudaMemcpyAsync(out, spos_ref + d.s_off, sizeof(float4) * d.s, cudaMemcpyDeviceToHost, stream_));
    }
    CUDA_TRY(cudaStreamSynchronize(stream_));
    if (out) {
        for (uint32_t i = 0; i < d.s; ++i) out[i].pressure = 0.f;   // static pressure is never written
    }
    if (bucket_starts) {
        CUDA_TRY(cudaMemcpy(bucket_starts, sstart_ref + d.sq_off, sizeof(uint32_t) * (d.s + 1ull), cudaMemcpyDeviceToHost));
        const uint32_t b0 = bucket_starts[0];
        for (uint32_t k = 0; k <= d.s; ++k) bucket_starts[k] -= b0;
    }
    return SPH_OK;
}

sph_status StepState::neighbour_stats(uint64_t out[kNeighbourStats])
{
    for (int k = 0; k < kNeighbourStats; ++k) out[k] = 0;
    if (tiles.empty()) return SPH_OK;
    unsigned long long* d = nullptr;
    sph_status st = dev_alloc(&d, kNeighbourStats);
    if (st != SPH_OK) return st;
    unsigned long long h[kNeighbourStats] = {};
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof h, stream_);
    if (e == cudaSuccess) {
        k_neighbour_stats<<<(unsigned)tiles.size(), kTileThreads, 0, stream_>>>(step_args(), d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, stream_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_last_error(std::string("neighbour statistics: ") + cudaGetErrorString(e));
        return SPH_ERR_CUDA;
    }
    for (int k = 0; k < kNeighbourStats; ++k) out[k] = h[k];
    return check_device_error();
}

sph_status StepState::read_buckets(uint32_t scene, uint32_t* bucket_starts, uint32_t* slot_ids)
{
    if (scene >= scenes.size()) return SPH_ERR_NOT_FOUND;
    const SceneDesc& d = scenes[scene];
    if (!d.n) return SPH_OK;
    CUDA_TRY(cudaStreamSynchronize(stream_));
    if (bucket_starts) {
        CUDA_TRY(cudaMemcpy(bucket_starts, start + d.q_off, sizeof(uint32_t) * (d.buckets + 1ull), cudaMemcpyDeviceToHost));
        const uint32_t b0 = bucket_starts[0];
        for (uint32_t k = 0; k <= d.buckets; ++k) bucket_starts[k] -= b0;
    }
    if (slot_ids) {
        std::vector<float4> tmp(d.n);
        CUDA_TRY(cudaMemcpy(tmp.data(), pos + d.p_off, sizeof(float4) * d.n, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < d.n; ++i) std::memcpy(&slot_ids[i], &tmp[i].w, 4);
    }
    return SPH_OK;
}

sph_status StepState::read_sort(uint32_t* keys, uint32_t* counts, uint32_t* starts, uint32_t* order)
{
    if (scenes.empty()) return SPH_ERR_NOT_INITIALIZED;
    const SceneDesc& d = scenes[0];
    CUDA_TRY(cudaStreamSynchronize(stream_));
    if (keys && d.n)   // keys are indexed by upload slot = input order
        CUDA_TRY(cudaMemcpy(keys, key + d.p_off, sizeof(uint32_t) * d.n, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> table(d.buckets + 1ull);
    CUDA_TRY(cudaMemcpy(table.data(), start + d.q_off, sizeof(uint32_t) * table.size(), cudaMemcpyDeviceToHost));
    const uint32_t b0 = table[0];
    for (auto& v : table) v -= b0;
    if (starts) std::memcpy(starts, table.data(), sizeof(uint32_t) * table.size());
    if (counts)
        for (uint32_t b = 0; b < d.buckets; ++b) counts[b] = table[b + 1] - table[b];
    if (order && d.n) {
        std::vector<float4> tmp(d.n);
        CUDA_TRY(cudaMemcpy(tmp.data(), pos + d.p_off, sizeof(float4) * d.n, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < d.n; ++i) std::memcpy(&order[i], &tmp[i].w, 4);
    }
    return check_device_error();
}

sph_status StepState::save_state()
{
    sph_status st;
    if (!saved_pos_ && (st = dev_alloc(&saved_pos_, cap_n_)) != SPH_OK) return st;
    if (!saved_vel_ && (st = dev_alloc(&saved_vel_, cap_n_)) != SPH_OK) return st;
    if (!saved_start_ && (st = dev_alloc(&saved_start_, cap_q_ + 1ull)) != SPH_OK) return st;
    if (!saved_tag_ && (st = dev_alloc(&saved_tag_, cap_n_)) != SPH_OK) return st;
    CUDA_TRY(cudaMemcpyAsync(saved_tag_, tag, sizeof(uint32_t) * cap_n_, cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(saved_pos_, pos, sizeof(float4) * cap_n_, cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(saved_vel_, vel, sizeof(float4) * cap_n_, cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(saved_start_, start, sizeof(uint32_t) * (cap_q_ + 1ull), cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(saved_nonfinite_, nonfinite, sizeof saved_nonfinite_, cudaMemcpyDeviceToHost, stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

sph_status StepState::restore_state()
{
    if (!saved_pos_ || !saved_vel_ || !saved_start_ || !saved_tag_) return SPH_ERR_NOT_INITIALIZED;
    CUDA_TRY(cudaMemcpyAsync(tag, saved_tag_, sizeof(uint32_t) * cap_n_, cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(pos, saved_pos_, sizeof(float4) * cap_n_, cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(vel, saved_vel_, sizeof(float4) * cap_n_, cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(start, saved_start_, sizeof(uint32_t) * (cap_q_ + 1ull), cudaMemcpyDeviceToDevice, stream_));
    CUDA_TRY(cudaMemcpyAsync(nonfinite, saved_nonfinite_, sizeof saved_nonfinite_, cudaMemcpyHostToDevice, stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

sph_status StepState::persistent_capacity(uint32_t* sms, uint32_t* per_sm)
{
    int s = 0, b = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, device_));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, persistent_kernel(exact_), kTileThreads, 0));
    *sms = (uint32_t)s;
    *per_sm = (uint32_t)std::max(b, 1);
    return SPH_OK;
}

}  // namespace sph
