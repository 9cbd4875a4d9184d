// sph_kernels.cuh -- the per-stage device routines of one SPH step.
//
// Each stage is a __device__ routine over one Tile (one CTA's slots of one
// scene), so the same code runs from a plain per-stage kernel and from the
// persistent fused step kernel.  Reference counterparts (SF =
// SPHFluidSimulation/source/SPH/Kernels/SPHFunctions.cpp):
//   hash_count_tile      SF:321-331  key + warp-aggregated bucket count
//   scan_tile            SF:227-294  single-pass decoupled-lookback scan
//   scatter_tile         SF:346-356  slot = bucket start + arrival rank
//   gather_tile          SF:332-345  rank inside the bucket by buffer tag + SoA move
//   density_tile         SF:358-501  27-bucket density / pressure pass
//   force_tile           SF:503-656  27-bucket force, integrate, rehash
//
// Data layout (struct of arrays, sorted by bucket every step):
//   pos[i] = (x, y, z, input index as bits)
//   vel[i] = (vx, vy, vz, pressure)       pressure written by the density pass
//   tag[i] = the particle's index in the reference's particle buffer
//
// The neighbour passes come in two arithmetic forms.  kExact = false (the
// default) fuses multiply-adds and divides by a reciprocal; kExact = true
// repeats the reference's operations one for one, so with the same visiting
// order its results are the reference's bits.
#pragma once
#include "sph_common.cuh"

namespace sph {

constexpr int kTileThreads = 128;          // slots per tile = threads per CTA

// Tuning knobs (compile-time; the defaults are the measured best on GB300).
// Minimum resident CTAs per SM requested from the register allocator for the
// two neighbour passes, and how many neighbours one round of the force and
// density-sum loops loads at once.
#ifndef SPH_DENSITY_MIN_CTAS
#define SPH_DENSITY_MIN_CTAS 7
#endif
#ifndef SPH_FORCE_MIN_CTAS
#define SPH_FORCE_MIN_CTAS 7
#endif
#ifndef SPH_NBR_BATCH
#define SPH_NBR_BATCH 4
#endif
constexpr int kScanThreads = kTileThreads;  // the scan runs inside the fused kernel too
constexpr int kScanItems = 8;              // per thread
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr uint32_t kSpinLimit = 1u << 21;  // bounded waits: ~1-2 s with backoff

struct StepArgs {
    const Tile* tiles;          // dynamic-particle tiles
    uint32_t num_tiles;
    const SceneDesc* scenes;
    float4* pos;                // sorted state
    float4* vel;
    float4* pos_tmp;            // unsorted output of the force pass
    float4* vel_tmp;
    uint32_t* key;              // local bucket of the new position, per tmp slot
    uint32_t* arrival;          // arrival rank inside the bucket, per tmp slot
    uint32_t* ptag;             // scatter slot -> buffer tag of the particle placed there
    uint32_t* tag;              // buffer tag per sorted slot (the reference's buffer index)
    uint32_t* count;            // bucket counters, zero between steps
    uint32_t* start;            // exclusive scan of count
    uint32_t scan_len;          // entries of count/start scanned
    unsigned long long* scan_status;
    uint32_t* scan_ticket;
    const float4* spos;         // static particles sorted for the neighbour passes
    const uint32_t* sstart;     // their bucket table (global scan, power-of-two buckets)
    const float4* spos_ref;     // static particles in the reference's own s-bucket order
    const uint32_t* sstart_ref; // its bucket table
    const float* tris;          // 9 floats per triangle
    const uint32_t* tri_cells;  // triangle cells: list starts per cell (+1)
    const uint32_t* tri_list;   // global triangle indices, increasing inside a cell
    const uint32_t* sbitmap;    // static-presence bitmaps of all scenes
    float4* accel;              // optional: acceleration per sorted slot (.w unused)
    uint32_t* err;              // device status word
    uint32_t* nonfinite;        // [0] current positions, [1] positions being written
    uint32_t* bar_count;        // grid barrier (persistent kernel only)
    uint32_t* bar_gen;
    uint32_t* nbr;              // neighbour lists [k][stride]
    uint32_t* snbr;
    uint32_t* ncount;
    uint32_t* tile_overflow;
    uint32_t nbr_stride;
};

// ---- small helpers ---------------------------------------------------------

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bit) { atomicOr(err, bit); }

// Adds 1 to counter[g] for every valid lane, one atomic per distinct g in the
// warp; returns this lane's arrival rank (the pre-increment value plus the
// number of lower lanes with the same g).
__device__ __forceinline__ uint32_t warp_aggregated_increment(uint32_t* counter, uint32_t g, bool valid)
{
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    uint32_t rank = 0;
    if (valid) {
        const unsigned peers = __match_any_sync(active, g);
        const int leader = __ffs(peers) - 1;
        const uint32_t lane = lane_id();
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(counter + g, (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        rank = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    }
    return rank;
}

// The 9 expanded coordinates of a cell's 3x3x3 neighbourhood: the Morton
// code of (c + d) is ex[dx] + ey[dy] + ez[dz] (SF:88-97 with the & 0x3FF
// mask, cells wrapping as unsigned like SF:386-395).  Kept in registers and
// picked with selects, so no local-memory array is needed.
struct Neighbourhood {
    uint32_t ex0, ex1, ex2, ey0, ey1, ey2, ez0, ez1, ez2;
};

__device__ __forceinline__ Neighbourhood neighbourhood(float x, float y, float z, float h)
{
    const uint32_t cx = cell_coord(x, h), cy = cell_coord(y, h), cz = cell_coord(z, h);
    Neighbourhood nb;
    nb.ex0 = expand_bits((cx - 1u) & 0x3FFu);
    nb.ex1 = expand_bits(cx & 0x3FFu);
    nb.ex2 = expand_bits((cx + 1u) & 0x3FFu);
    nb.ey0 = expand_bits((cy - 1u) & 0x3FFu) * 2u;
    nb.ey1 = expand_bits(cy & 0x3FFu) * 2u;
    nb.ey2 = expand_bits((cy + 1u) & 0x3FFu) * 2u;
    nb.ez0 = expand_bits((cz - 1u) & 0x3FFu) * 4u;
    nb.ez1 = expand_bits(cz & 0x3FFu) * 4u;
    nb.ez2 = expand_bits((cz + 1u) & 0x3FFu) * 4u;
    return nb;
}

__device__ __forceinline__ uint32_t pick3(int k, uint32_t v0, uint32_t v1, uint32_t v2)
{
    return k == 0 ? v0 : (k == 1 ? v1 : v2);
}

// Morton code of neighbour cell (a, b, c) in {0,1,2}^3, x outermost as in
// the reference's loops (SF:392-395).
__device__ __forceinline__ uint32_t neighbour_hash(const Neighbourhood& nb, int a, int b, int c)
{
    return pick3(a, nb.ex0, nb.ex1, nb.ex2) + pick3(b, nb.ey0, nb.ey1, nb.ey2) + pick3(c, nb.ez0, nb.ez1, nb.ez2);
}

// RandomDirection (SF:140-155), used only for coincident particles, with the
// reference C++ build's conversions: sin of the float product in double, the
// fraction by modf (keeping the sign of its argument, so noise lies in
// (-1, 1) and z in (-3, 1): for z < -1 the square root is NaN, as in the
// reference), then sin, cos and the root rounded to float and multiplied in
// float (SF:151-154).  Every operation is rounded on its own: no contraction.
__device__ __noinline__ inline float3 random_direction(float x)
{
    const double v = __dmul_rn(sin((double)__fmul_rn(x, 112.9898f)), (double)43758.5453f);
    const float noise = (float)__dsub_rn(v, trunc(v));
    const float theta = __fmul_rn(__fmul_rn(noise, 2.0f), 3.1415f);
    const float z = __fsub_rn(__fmul_rn(noise, 2.0f), 1.0f);
    const float sn = (float)sin((double)theta);
    const float cs = (float)cos((double)theta);
    const float z2 = (float)__dsqrt_rn((double)__fsub_rn(1.0f, __fmul_rn(z, z)));
    return make_float3(__fmul_rn(z2, cs), __fmul_rn(z2, sn), z);
}

// ClosestPointOnTriangle + CalculateTriangleForce (SF:156-223).
__device__ __noinline__ inline float3 triangle_force(float3 p, const float* tri)
{
    const float3 a = make_float3(tri[0], tri[1], tri[2]);
    const float3 b = make_float3(tri[3], tri[4], tri[5]);
    const float3 c = make_float3(tri[6], tri[7], tri[8]);
    auto sub = [](float3 u, float3 v) { return make_float3(u.x - v.x, u.y - v.y, u.z - v.z); };
    auto dot = [](float3 u, float3 v) { return __fadd_rn(__fadd_rn(__fmul_rn(u.x, v.x), __fmul_rn(u.y, v.y)), __fmul_rn(u.z, v.z)); };
    auto axpy = [](float3 o, float3 u, float s) { return make_float3(__fadd_rn(o.x, __fmul_rn(u.x, s)), __fadd_rn(o.y, __fmul_rn(u.y, s)), __fadd_rn(o.z, __fmul_rn(u.z, s))); };
    float3 q;
    const float3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const float d1 = dot(ab, ap), d2 = dot(ac, ap);
    const float3 bp = sub(p, b);
    const float d3 = dot(ab, bp), d4 = dot(ac, bp);
    const float3 cp = sub(p, c);
    const float d5 = dot(ab, cp), d6 = dot(ac, cp);
    const float vc = __fsub_rn(__fmul_rn(d1, d4), __fmul_rn(d3, d2));
    const float vb = __fsub_rn(__fmul_rn(d5, d2), __fmul_rn(d1, d6));
    const float va = __fsub_rn(__fmul_rn(d3, d6), __fmul_rn(d5, d4));
    if (d1 <= 0.f && d2 <= 0.f) q = a;
    else if (d3 >= 0.f && d4 <= d3) q = b;
    else if (d6 >= 0.f && d5 <= d6) q = c;
    else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) q = axpy(a, ab, __fdiv_rn(d1, __fsub_rn(d1, d3)));
    else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) q = axpy(a, ac, __fdiv_rn(d2, __fsub_rn(d2, d6)));
    else if (va <= 0.f && __fsub_rn(d4, d3) >= 0.f && __fsub_rn(d5, d6) >= 0.f) {
        const float e = __fsub_rn(d4, d3);
        q = axpy(b, sub(c, b), __fdiv_rn(e, __fadd_rn(e, __fsub_rn(d5, d6))));
    } else {
        const float denom = __fdiv_rn(1.f, __fadd_rn(__fadd_rn(va, vb), vc));
        q = axpy(axpy(a, ab, __fmul_rn(vb, denom)), ac, __fmul_rn(vc, denom));
    }
    const float3 to = sub(q, p);
    const float dist = __fsqrt_rn(dot(to, to));
    if (dist > kTriangleReach) return make_float3(0.f, 0.f, 0.f);
    const float t = __fsub_rn(__fdiv_rn(1.f, __fdiv_rn(dist, kTriangleReach)), 1.f);
    const float amp = __fmul_rn(t, t);
    float3 dir = make_float3(__fdiv_rn(-to.x, dist), __fdiv_rn(-to.y, dist), __fdiv_rn(-to.z, dist));
    return make_float3(__fmul_rn(__fmul_rn(dir.x, amp), 50.f), __fmul_rn(__fmul_rn(dir.y, amp), 50.f),
                       __fmul_rn(__fmul_rn(dir.z, amp), 50.f));
}

// ---- stage: hash + count ---------------------------------------------------

// True when all three coordinates are finite.  A NaN or infinite coordinate
// makes every distance NaN, and the reference keeps NaN distances: its tests
// skip a neighbour only when distSqr > h^2 (SF:447-448, 488-489, 571-572,
// 605-606) and its
// kernels return 0 only when r >= h (SF:119-139), so a non-finite particle
// is a neighbour of everything its buckets hold and turns their sums NaN.
__device__ __forceinline__ bool finite3(const float4& p)
{
    return isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
}

// key[i] = GetHash(GetCell(pos[i])) % buckets; count[q_off + key]++ with one
// atomic per distinct key per warp; arrival[i] = rank among that key's adds.
__device__ __forceinline__ void hash_count_tile(const Tile& tile, const SceneDesc* scenes, const float4* pos,
                                                uint32_t* key, uint32_t* arrival, uint32_t* count,
                                                uint32_t* nonfinite = nullptr)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    const bool valid = i < tile.end;
    uint32_t g = 0, k = 0;
    if (valid) {
        const float4 p = pos[i];
        k = fast_mod(cell_hash(p.x, p.y, p.z, sc.h), sc.fm_b);
        g = sc.q_off + k;
        if (nonfinite && !finite3(p)) atomicOr(nonfinite, 1u);
    }
    const uint32_t r = warp_aggregated_increment(count, g, valid);
    if (valid) {
        key[i] = k;
        arrival[i] = r;
    }
}

// ---- stage: exclusive scan (decoupled look-back) ---------------------------
//
// Merrill & Garland, "Single-pass Parallel Prefix Scan with Decoupled
// Look-back" (NVIDIA TR, 2016).  Tile ids come from a ticket counter so a
// tile only ever waits on tiles already claimed by running CTAs.  Status
// word: bits 32-33 = 1 aggregate, 2 inclusive prefix; low 32 bits = value.
// Every wait is bounded; on expiry the error word is set and the scan
// finishes with the value it has (the host reports SPH_ERR_DEVICE_TIMEOUT).
// Writes start[i] = sum(count[0..i)), then zeroes count[i].

struct ScanSmem {
    uint4 items[kScanThreads * kScanItems / 4];
    uint32_t warp_sums[kScanThreads / 32];
    uint32_t tile;
    uint32_t exclusive;
};

__device__ __forceinline__ unsigned long long load_status(const unsigned long long* p)
{
    return *(const volatile unsigned long long*)p;
}

__device__ inline void scan_tile(uint32_t tile, uint32_t* count, uint32_t* start, uint32_t len,
                          unsigned long long* status, uint32_t* err, ScanSmem& sm)
{
    const uint32_t base = tile * (uint32_t)kScanTile;
    const uint32_t t = threadIdx.x;
    // striped vector loads into shared memory
#pragma unroll
    for (int k = 0; k < kScanItems / 4; ++k) {
        const uint32_t v = (uint32_t)k * kScanThreads + t;        // uint4 index in tile
        const uint32_t e = base + v * 4u;
        uint4 q;
        if (e + 4u <= len) {
            q = *reinterpret_cast<const uint4*>(count + e);
        } else {
            q.x = e + 0u < len ? count[e + 0u] : 0u;
            q.y = e + 1u < len ? count[e + 1u] : 0u;
            q.z = e + 2u < len ? count[e + 2u] : 0u;
            q.w = e + 3u < len ? count[e + 3u] : 0u;
        }
        sm.items[v] = q;
    }
    __syncthreads();
    // each thread owns kScanItems consecutive items
    uint32_t vals[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems / 4; ++k) {
        const uint4 q = sm.items[t * (kScanItems / 4) + k];
        vals[4 * k + 0] = q.x; vals[4 * k + 1] = q.y; vals[4 * k + 2] = q.z; vals[4 * k + 3] = q.w;
        sum += q.x + q.y + q.z + q.w;
    }
    // block-wide exclusive scan of the per-thread sums
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane_id() >= (uint32_t)o) incl += y;
    }
    const uint32_t warp = t >> 5;
    if (lane_id() == 31u) sm.warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane_id() < kScanThreads / 32 ? sm.warp_sums[lane_id()] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane_id() >= (uint32_t)o) wi += y;
        }
        const uint32_t aggregate = __shfl_sync(0xffffffffu, wi, kScanThreads / 32 - 1);
        if (lane_id() < kScanThreads / 32) sm.warp_sums[lane_id()] = wi - w;   // exclusive per warp
        // publish and look back
        uint32_t exclusive = 0;
        if (tile == 0) {
            if (lane_id() == 0)
                atomicExch(&status[0], (2ull << 32) | (unsigned long long)aggregate);
        } else {
            if (lane_id() == 0)
                atomicExch(&status[tile], (1ull << 32) | (unsigned long long)aggregate);
            int64_t pred = (int64_t)tile - 1;
            uint32_t spins = 0;
            bool timed_out = false;
            while (true) {
                const int64_t idx = pred - (int64_t)lane_id();
                unsigned long long s = idx >= 0 ? load_status(&status[idx]) : (2ull << 32);
                uint32_t flag = (uint32_t)(s >> 32) & 3u;
                if (__any_sync(0xffffffffu, flag == 0u) && !timed_out) {
                    if (++spins > kSpinLimit) {
                        timed_out = true;
                        if (lane_id() == 0) set_error(err, DEV_ERR_SCAN_TIMEOUT);
                    } else {
                        __nanosleep(spins < 64 ? 32 : 256);
                    }
                    continue;
                }
                if (flag == 0u) { s = (2ull << 32); flag = 2u; }          // timed out: stop here
                const unsigned prefix_mask = __ballot_sync(0xffffffffu, flag == 2u);
                const uint32_t value = (uint32_t)s;
                if (prefix_mask) {
                    const int first = __ffs(prefix_mask) - 1;             // nearest inclusive prefix
                    uint32_t contrib = (int)lane_id() <= first ? value : 0u;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
                    exclusive += contrib;
                    break;
                }
                uint32_t contrib = value;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
                exclusive += contrib;
                pred -= 32;
            }
            if (lane_id() == 0)
                atomicExch(&status[tile], (2ull << 32) | (unsigned long long)(exclusive + aggregate));
        }
        if (lane_id() == 0) sm.exclusive = exclusive;
    }
    __syncthreads();
    uint32_t run = sm.exclusive + sm.warp_sums[warp] + (incl - sum);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t c = vals[k];
        vals[k] = run;
        run += c;
    }
    // write back through shared memory (striped, vectorised)
#pragma unroll
    for (int k = 0; k < kScanItems / 4; ++k)
        sm.items[t * (kScanItems / 4) + k] = make_uint4(vals[4 * k], vals[4 * k + 1], vals[4 * k + 2], vals[4 * k + 3]);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems / 4; ++k) {
        const uint32_t v = (uint32_t)k * kScanThreads + t;
        const uint32_t e = base + v * 4u;
        const uint4 q = sm.items[v];
        if (e + 4u <= len) {
            *reinterpret_cast<uint4*>(start + e) = q;
            *reinterpret_cast<uint4*>(count + e) = make_uint4(0u, 0u, 0u, 0u);
        } else {
            if (e + 0u < len) { start[e + 0u] = q.x; count[e + 0u] = 0u; }
            if (e + 1u < len) { start[e + 1u] = q.y; count[e + 1u] = 0u; }
            if (e + 2u < len) { start[e + 2u] = q.z; count[e + 2u] = 0u; }
        }
    }
    __syncthreads();
}

// ---- stage: scatter (arrival order) ----------------------------------------
//
// Every particle lands on slot start + arrival rank and leaves its buffer tag
// there: tag_src[j] when the sort carries tags, else the source slot j.

// What the gather writes to tag_dst.
enum TagAssign : uint32_t {
    kTagNone = 0,    // no tags (static sorts)
    kTagSlot = 1,    // the new slot inside the scene (the initial sort)
    kTagKeep = 2,    // the source tag (a write between steps)
    kTagStep = 3,    // per scene: the new slot on a reordering step, else the source tag
};

__device__ __forceinline__ void scatter_tile(const Tile& tile, const SceneDesc* scenes, const uint32_t* key,
                                             const uint32_t* arrival, const uint32_t* start,
                                             const uint32_t* tag_src, uint32_t* ptag, uint32_t* err)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    if (i >= tile.end) return;
    const uint32_t delta = sc.p_off - start[sc.q_off];
    const uint32_t slot = start[sc.q_off + key[i]] + delta + arrival[i];
    if (slot - sc.p_off >= sc.n) { set_error(err, DEV_ERR_SLOT_RANGE); return; }
    ptag[slot] = tag_src ? tag_src[i] : i;
}

// ---- stage: stable gather --------------------------------------------------
//
// Inside a bucket the members are ordered by decreasing tag: source slot j
// moves to bucket start + (number of members with a larger tag).  That is
// the order every counting sort of the reference produces, which fills each
// bucket from its end while it walks the buffer upwards
// (SimulationEngine.h:96-97, SF:332-356 with SimulationEngineCPU.cpp:288-316),
// so the neighbour passes visit a bucket's members exactly as the reference
// does.  Tags are the reference's buffer indices: fixed between reorders,
// renumbered to the new slot by a reordering step.  Buckets hold a handful
// of particles, so the rank loop reads a few words from L1.
constexpr uint32_t kStableRankLimit = 8192;   // larger buckets keep arrival order

__device__ __forceinline__ void gather_tile(const Tile& tile, const SceneDesc* scenes, const uint32_t* key,
                                            const uint32_t* arrival, const uint32_t* ptag, const uint32_t* start,
                                            const float4* pos_src, const float4* vel_src, float4* pos_dst,
                                            float4* vel_dst, uint32_t* tag_dst, uint32_t assign, uint32_t* err,
                                            const float4* accel_src = nullptr, float4* accel_dst = nullptr,
                                            const uint32_t* tag_keep = nullptr)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t j = tile.begin + threadIdx.x;
    if (j >= tile.end) return;
    const uint32_t delta = sc.p_off - start[sc.q_off];
    const uint32_t g = sc.q_off + key[j];
    const uint32_t b0 = start[g] + delta;
    const uint32_t e0 = start[g + 1] + delta;
    if (b0 - sc.p_off > sc.n || e0 - sc.p_off > sc.n || e0 < b0) { set_error(err, DEV_ERR_BUCKET_RANGE); return; }
    const uint32_t mine_at = b0 + arrival[j];
    if (mine_at >= e0) { set_error(err, DEV_ERR_SLOT_RANGE); return; }
    const uint32_t mine = ptag[mine_at];
    uint32_t rank = 0;
    if (e0 - b0 <= kStableRankLimit) {
        for (uint32_t t = b0; t < e0; ++t) rank += (ptag[t] > mine) ? 1u : 0u;
    } else {
        rank = arrival[j];
    }
    const uint32_t dst = b0 + rank;
    if (dst >= e0) { set_error(err, DEV_ERR_SLOT_RANGE); return; }
    pos_dst[dst] = pos_src[j];
    vel_dst[dst] = vel_src[j];
    if (accel_src) accel_dst[dst] = accel_src[j];
    if (assign != kTagNone) {
        const bool renumber = assign == kTagSlot || (assign == kTagStep && sc.reorder);
        // tag_keep: the ranking key is not the tag (a write ranks by the slot
        // each particle had before it); the tag comes from the source slot
        tag_dst[dst] = renumber ? dst - sc.p_off : (tag_keep ? tag_keep[j] : mine);
    }
}

// Squared distance with a fixed rounding sequence, so every kernel that
// inlines it produces the same bits.
__device__ __forceinline__ float dist2(const float4& q, const float4& p)
{
    const float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// ---- stage: density / pressure ---------------------------------------------
//
// UpdateParticlePressure (SF:358-501): over the 27 buckets of the cell
// neighbourhood (x outermost, bucket ids repeating where cells collide, as in
// the reference), sum (h - r)^3 over dynamic neighbours (self skipped) and
// static neighbours within h; rho = selfDensity + (sum_d m + sum_s m) C and
// p = k (rho - rho0), stored in vel.w.
//
// The pass runs in two loops.  The test loop visits every candidate and
// appends the slot of each one with r^2 <= h^2 to the particle's neighbour
// list (column layout nbr[k * stride + i]).  The sum loop then walks the list,
// so the square root and the kernel polynomial run once per neighbour
// instead of under divergence for every candidate.  The force pass reuses the
// same list.  A particle with more than kMaxNbr dynamic or kMaxSNbr static
// neighbours is flagged (kOverflow) and summed by re-walking its buckets.
//
// Neighbour cells whose box lies farther than h from the particle hold no
// neighbour and are skipped, provided the 27 bucket ids are distinct (their
// Morton codes span less than the bucket count); otherwise all 27 are walked.

// L2 residency hints for the neighbour lists (PTX createpolicy and
// .L2::cache_hint).  The density pass writes the lists and the force pass of
// the same step reads each entry once: the stores ask L2 to keep the lines
// (evict_last), the force pass's loads let them go (evict_first).
__device__ __forceinline__ uint64_t l2_policy_keep()
{
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ uint64_t l2_policy_drop()
{
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ void store_list(uint32_t* a, uint32_t v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(a), "r"(v), "l"(pol) : "memory");
}

__device__ __forceinline__ uint32_t load_list(const uint32_t* a, uint64_t pol)
{
    uint32_t v;
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

constexpr uint32_t kMaxNbr = 96;        // dynamic neighbours listed per particle
constexpr uint32_t kMaxSNbr = 48;       // static neighbours listed per particle
constexpr uint32_t kOverflow = 0xFFFFu;

// Row length of the neighbour lists: the slot capacity rounded up to 32, so
// a row's entries for 32 slots starting at a multiple of 32 fill one
// 128-byte line.
__host__ __device__ __forceinline__ uint32_t list_stride(uint32_t cap_n) { return (cap_n + 31u) & ~31u; }

struct NbrArgs {
    uint32_t* nbr;         // [kMaxNbr][stride]
    uint32_t* snbr;        // [kMaxSNbr][stride]
    uint32_t* ncount;      // dynamic count | static count << 16
    uint32_t* tile_overflow;
    uint32_t stride;
    const uint32_t* nonfinite;   // non-zero: some current position is not finite
};

__device__ __forceinline__ float pick3f(int k, float v0, float v1, float v2)
{
    return k == 0 ? v0 : (k == 1 ? v1 : v2);
}

__device__ __forceinline__ uint32_t span3(uint32_t a, uint32_t b, uint32_t c)
{
    return max(max(a, b), c) - min(min(a, b), c);
}

// Squared distances from the particle to the boxes of its neighbour cells
// along one axis: offset -1, 0, +1.  Conservative (cull threshold carries a
// relative margin) and disabled far from the origin where the float cell
// corner is inexact.
struct CellBox {
    float x0, x2, y0, y2, z0, z2;   // squared face distances (offset 0 -> 0)
    bool ok;
};

__device__ __forceinline__ CellBox cell_box(const float4& p, float h)
{
    CellBox b;
    // the unwrapped cell, exact as a float while |cell| < 2^22 (NaN: not ok)
    const float cx = floorf(p.x / h), cy = floorf(p.y / h), cz = floorf(p.z / h);
    b.ok = fabsf(cx) < 4194304.f && fabsf(cy) < 4194304.f && fabsf(cz) < 4194304.f;
    const float fx = p.x - cx * h, fy = p.y - cy * h, fz = p.z - cz * h;
    const float gx = fmaxf(h - fx, 0.f), gy = fmaxf(h - fy, 0.f), gz = fmaxf(h - fz, 0.f);
    const float ax = fmaxf(fx, 0.f), ay = fmaxf(fy, 0.f), az = fmaxf(fz, 0.f);
    b.x0 = ax * ax; b.x2 = gx * gx;
    b.y0 = ay * ay; b.y2 = gy * gy;
    b.z0 = az * az; b.z2 = gz * gz;
    return b;
}

__device__ __forceinline__ uint32_t nb_span(const Neighbourhood& nb)
{
    return span3(nb.ex0, nb.ex1, nb.ex2) + span3(nb.ey0, nb.ey1, nb.ey2) + span3(nb.ez0, nb.ez1, nb.ez2);
}

// Distance from its square.  The reference's arithmetic takes the correctly
// rounded root; the fast form multiplies r^2 by the hardware reciprocal
// square root (rsqrtf, within 2 ulp), whose value also scales the direction
// in the force pass.  r^2 = 0 gives 0 and NaN stays NaN in both.
template <bool kExact>
__device__ __forceinline__ float root_of(float r2, float rinv)
{
    return kExact ? __fsqrt_rn(r2) : (r2 == 0.f ? 0.f : __fmul_rn(r2, rinv));
}

template <bool kExact>
__device__ __forceinline__ float w0_of(float r2, float h)
{
    const float r = root_of<kExact>(r2, kExact ? 0.f : rsqrtf(r2));
    const float w = __fsub_rn(h, r);
    return r >= h ? 0.f : __fmul_rn(__fmul_rn(w, w), w);   // NaN stays NaN (SF:119-125)
}

// Squared distance in the reference's own arithmetic: dir = q - p, then
// dot(dir, dir) summed left to right with no contraction (SF:437-438 and the
// Vec3 dot product).  dist2() above fuses the two adds; both round each step.
__device__ __forceinline__ float dist2_ref(const float4& q, const float4& p)
{
    const float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

template <bool kExact>
__device__ __forceinline__ float pair_r2(const float4& q, const float4& p)
{
    return kExact ? dist2_ref(q, p) : dist2(q, p);
}

// Static neighbour list entries: an index into the neighbour-pass table, or,
// with bit 31 set, into the reference's own s-bucket table.  Particles whose
// 27 static buckets may repeat walk that table itself, visiting every bucket
// as the reference does, so a static particle reached through two cells is
// listed twice, in the reference's order.
constexpr uint32_t kRefTableBit = 1u << 31;

// The static tables the neighbour passes read.
struct StaticTables {
    const float4* spos;         // neighbour-pass table: sorted statics, w = cell Morton code
    const uint32_t* sstart;
    const float4* spos_ref;     // the reference's table (hash % s)
    const uint32_t* sstart_ref;
    const uint32_t* sbitmap;    // static-presence bitmaps
};

// What a neighbour walk of one particle needs to know about its 27 cells.
struct Walk {
    Neighbourhood nb;
    CellBox box;
    bool cull_d;        // dynamic buckets are distinct: cells beyond h may be skipped
    bool dup_s;         // the reference's static buckets may repeat
    bool near_static;   // a static particle lies within one cell
    bool ref_walk;      // statics walk the reference's own table (dup_s)
};

// `nonfinite_seen`: some particle of the state has a non-finite coordinate.
// Such a particle is every visited particle's neighbour (finite3), wherever
// its bucket lies, so cells beyond h are not skipped while one exists; and a
// non-finite particle itself walks every bucket the reference walks: all 27
// dynamic ones and the reference's own static table.
template <bool kExact>
__device__ __forceinline__ Walk make_walk(const SceneDesc& sc, const float4& p, const uint32_t* sbitmap,
                                          bool nonfinite_seen)
{
    Walk w;
    const bool fin = finite3(p);
    w.nb = neighbourhood(p.x, p.y, p.z, sc.h);
    w.box = cell_box(p, sc.h);
    const uint32_t span = nb_span(w.nb);
    w.cull_d = w.box.ok && span < sc.buckets && !nonfinite_seen;
    w.dup_s = span >= sc.s;
    const uint32_t own = (w.nb.ex1 + w.nb.ey1 + w.nb.ez1) & sc.sbm_mask;
    w.near_static = sc.s && (!fin || ((__ldg(sbitmap + sc.sbm_off + (own >> 5)) >> (own & 31u)) & 1u));
    w.ref_walk = w.near_static && (w.dup_s || !fin);
    return w;
}

// Visits the neighbours of slot i within h in the reference's order: the 27
// cells x outermost (SF:392-395), each cell's dynamic bucket members in
// bucket order (on_dyn(j, q, r2)), then its static ones (on_static(entry, q,
// r2)).  Dynamic and static sums are separate in the reference, so only the
// order inside each kind matters.  Cells whose box lies beyond h are skipped
// when their bucket cannot hold another visited cell's particles.
// on_cell(members) follows each cell's dynamic bucket with the number of
// candidates tested there (0 when skipped); every lane of a warp calls it
// 27 times in the same order.  kDyn = false walks the static buckets only.
template <bool kExact, bool kDyn = true, typename FD, typename FS, typename FC>
__device__ __forceinline__ void walk_neighbours_cells(const SceneDesc& sc, uint32_t i, const float4& p,
                                                      const Walk& w, const float4* __restrict__ pos,
                                                      const uint32_t* __restrict__ start, const StaticTables& st,
                                                      FD&& on_dyn, FS&& on_static, FC&& on_cell)
{
    const float h2 = sc.h2;
    const float cull2 = __fmul_rn(h2, 1.0001f);
    const uint32_t delta = kDyn ? sc.p_off - __ldg(start + sc.q_off) : 0u;
    uint32_t sdelta = 0;
    if (w.near_static)
        sdelta = sc.s_off - (w.ref_walk ? __ldg(st.sstart_ref + sc.sq_off) : __ldg(st.sstart + sc.sf_off));
#pragma unroll 1
    for (int a = 0; a < 3; ++a)
#pragma unroll 1
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float bd2 = pick3f(a, w.box.x0, 0.f, w.box.x2) + pick3f(b, w.box.y0, 0.f, w.box.y2) +
                                  pick3f(c, w.box.z0, 0.f, w.box.z2);
                const bool far = bd2 > cull2;
                const uint32_t hsh = neighbour_hash(w.nb, a, b, c);
                uint32_t members = 0;
                if (kDyn && !(far && w.cull_d)) {
                    const uint32_t bk = sc.q_off + fast_mod(hsh, sc.fm_b);
                    const uint32_t beg = max(__ldg(start + bk) + delta, sc.p_off);
                    const uint32_t end = min(__ldg(start + bk + 1) + delta, sc.p_off + sc.n);
                    for (uint32_t j = beg; j < end; ++j) {
                        const float4 q = __ldg(pos + j);
                        const float r2 = pair_r2<kExact>(q, p);
                        if (!(r2 > h2) && j != i) on_dyn(j, q, r2);
                    }
                    members = end > beg ? end - beg : 0u;
                }
                if (kDyn) on_cell(members);
                if (!w.near_static) continue;
                if (w.ref_walk) {
                    // SF:454-490: bucket hash % s of the reference's table, every member
                    const uint32_t sb = sc.sq_off + fast_mod(hsh, sc.fm_s);
                    const uint32_t sbeg = max(__ldg(st.sstart_ref + sb) + sdelta, sc.s_off);
                    const uint32_t send = min(__ldg(st.sstart_ref + sb + 1) + sdelta, sc.s_off + sc.s);
                    for (uint32_t j = sbeg; j < send; ++j) {
                        const float4 q = __ldg(st.spos_ref + j);
                        const float r2 = pair_r2<kExact>(q, p);
                        if (!(r2 > h2)) on_static(j | kRefTableBit, q, r2);
                    }
                } else if (!(far && w.box.ok)) {
                    const uint32_t sb = sc.sf_off + fast_mod(hsh, sc.fm_sf);
                    const uint32_t sbeg = max(__ldg(st.sstart + sb) + sdelta, sc.s_off);
                    const uint32_t send = min(__ldg(st.sstart + sb + 1) + sdelta, sc.s_off + sc.s);
                    for (uint32_t j = sbeg; j < send; ++j) {
                        const float4 q = __ldg(st.spos + j);
                        // statics carry their cell's Morton code: only this cell's count
                        if (__float_as_uint(q.w) != hsh) continue;
                        const float r2 = pair_r2<kExact>(q, p);
                        if (!(r2 > h2)) on_static(j, q, r2);
                    }
                }
            }
}

template <bool kExact, typename FD, typename FS>
__device__ __forceinline__ void walk_neighbours(const SceneDesc& sc, uint32_t i, const float4& p, const Walk& w,
                                                const float4* __restrict__ pos, const uint32_t* __restrict__ start,
                                                const StaticTables& st, FD&& on_dyn, FS&& on_static)
{
    walk_neighbours_cells<kExact>(sc, i, p, w, pos, start, st, on_dyn, on_static, [](uint32_t) {});
}

// Position of a static list entry.
__device__ __forceinline__ float4 static_entry_pos(uint32_t e, const StaticTables& st)
{
    return (e & kRefTableBit) ? __ldg(st.spos_ref + (e & ~kRefTableBit)) : __ldg(st.spos + e);
}

constexpr int kDensityThreads = kTileThreads;   // one home slot per thread

// Sum of (h - r)^3 over the first cnt entries of slot i's neighbour list, in
// list order.  Four neighbours per round, their loads issued together; the
// next round's entries load while this round's positions arrive.
template <bool kExact>
__device__ __forceinline__ float sum_list(const NbrArgs& nl, uint32_t i, uint32_t cnt, const float4* __restrict__ pos,
                                          const float4& p, float h)
{
    const uint32_t stride = nl.stride;
    float sum_d = 0.f;
    const uint32_t* lp = nl.nbr + i;
    uint32_t m = 0;
    uint32_t n0 = 0, n1 = 0, n2 = 0, n3 = 0;
    if (SPH_NBR_BATCH == 4 && m + 4 <= cnt) {
        n0 = lp[0]; n1 = lp[stride]; n2 = lp[2 * (size_t)stride]; n3 = lp[3 * (size_t)stride];
    }
    for (; SPH_NBR_BATCH == 4 && m + 4 <= cnt; m += 4, lp += 4 * (size_t)stride) {
        const uint32_t j0 = n0, j1 = n1, j2 = n2, j3 = n3;
        if (m + 8 <= cnt) {
            const uint32_t* ln = lp + 4 * (size_t)stride;
            n0 = ln[0]; n1 = ln[stride]; n2 = ln[2 * (size_t)stride]; n3 = ln[3 * (size_t)stride];
        }
        const float4 q0 = __ldg(pos + j0), q1 = __ldg(pos + j1), q2 = __ldg(pos + j2), q3 = __ldg(pos + j3);
        sum_d = __fadd_rn(sum_d, w0_of<kExact>(pair_r2<kExact>(q0, p), h));
        sum_d = __fadd_rn(sum_d, w0_of<kExact>(pair_r2<kExact>(q1, p), h));
        sum_d = __fadd_rn(sum_d, w0_of<kExact>(pair_r2<kExact>(q2, p), h));
        sum_d = __fadd_rn(sum_d, w0_of<kExact>(pair_r2<kExact>(q3, p), h));
    }
    for (; m < cnt; ++m, lp += stride) sum_d = __fadd_rn(sum_d, w0_of<kExact>(pair_r2<kExact>(__ldg(pos + *lp), p), h));
    return sum_d;
}

// One slot per thread.  (Two home particles per thread sharing candidate
// loads measured 3x slower on GB300: the extra registers cost more occupancy
// than the loads saved.)
template <bool kExact>
__device__ __forceinline__ void density_tile(uint32_t tile_index, const Tile& tile, uint32_t lane,
                                             const SceneDesc* scenes, const float4* __restrict__ pos,
                                             float4* __restrict__ vel, const uint32_t* __restrict__ start,
                                             const StaticTables& st, const NbrArgs& nl)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + lane;
    if (i >= tile.end) return;
    const float h = sc.h;
    const float4 p = pos[i];
    const Walk w = make_walk<kExact>(sc, p, st.sbitmap, *nl.nonfinite != 0u);
    const uint32_t stride = nl.stride;
    uint32_t cnt = 0, scnt = 0;
    const uint64_t keep = l2_policy_keep();
    walk_neighbours<kExact>(
        sc, i, p, w, pos, start, st,
        [&](uint32_t j, const float4&, float) {
            if (cnt < kMaxNbr) store_list(nl.nbr + (size_t)cnt * stride + i, j, keep);
            ++cnt;
        },
        [&](uint32_t e, const float4&, float) {
            if (scnt < kMaxSNbr) store_list(nl.snbr + (size_t)scnt * stride + i, e, keep);
            ++scnt;
        });
    float sum_d = 0.f, sum_s = 0.f;
    const bool overflow = cnt > kMaxNbr || scnt > kMaxSNbr;
    if (!overflow) {
        sum_d = sum_list<kExact>(nl, i, cnt, pos, p, h);
        const uint32_t* lp = nl.snbr + i;
        for (uint32_t k = 0; k < scnt; ++k, lp += stride)
            sum_s = __fadd_rn(sum_s, w0_of<kExact>(pair_r2<kExact>(static_entry_pos(*lp, st), p), h));
    } else {
        // overflow: walk the cells again, summing directly
        walk_neighbours<kExact>(
            sc, i, p, w, pos, start, st,
            [&](uint32_t, const float4&, float r2) { sum_d = __fadd_rn(sum_d, w0_of<kExact>(r2, h)); },
            [&](uint32_t, const float4&, float r2) { sum_s = __fadd_rn(sum_s, w0_of<kExact>(r2, h)); });
        atomicOr(nl.tile_overflow + tile_index, 1u);   // cleared by the overflow force pass
    }
    nl.ncount[i] = overflow ? (kOverflow | (kOverflow << 16)) : (cnt | (scnt << 16));
    // SF:497-498
    const float rho = __fadd_rn(sc.self_density,
                                __fmul_rn(__fadd_rn(__fmul_rn(sum_d, sc.mass), __fmul_rn(sum_s, sc.mass)), sc.kc));
    const float pressure = __fmul_rn(sc.gas, __fsub_rn(rho, sc.rho0));
    reinterpret_cast<float*>(vel + i)[3] = pressure;
}

// ---- density: the group walk -------------------------------------------------
//
// The same pass, bit for bit, organised around cells instead of slots.  All
// slots of one cell (one Morton code) have the same 27 neighbour buckets, so
// their candidates are one sequence: the members of the 27 buckets in the
// walk's order (x outermost, bucket order inside a bucket).  A warp takes its
// 32 slots cell by cell ("groups"):
//   1. lanes 0..26 look up one bucket each and a warp scan places them; the
//      candidates' slots go to shared memory and their positions to
//      registers, 32 candidates per register slot;
//   2. for each home of the group, every lane tests its candidates against
//      the home and a ballot per register slot records the hits: one test
//      per candidate and lane, no lane waits at a bucket end;
//   3. each home's lane decodes its hit bits in candidate order, appending
//      its neighbour list and summing (h - r)^3 in that order, as
//      density_tile does.
// The hits are those of density_tile's test (same r^2 arithmetic, same
// operands; the cells it skips hold none), so the lists, counts and sums are
// density_tile's.  Where the 27 buckets may repeat, a repeated bucket is a
// repeated candidate, as in density_tile, and the home itself is skipped at
// every place it appears.  Slots whose cell holds more than kGroupSlots * 32
// candidates, and slots at a non-finite position (whose test passes every
// candidate, padding included), run density_tile itself; statics are walked
// per slot.
constexpr uint32_t kGroupSlots = 8;     // candidate registers per lane: 256 candidates per group
// Candidate slots one warp holds in shared memory: a warp's groups hold
// about 27 x (32 + cell occupancy) candidates, about 1080 at 8 slots per
// cell; past the limit the waiting homes are finished first (step 3).
constexpr uint32_t kWarpCand = 1280;

struct GroupSmem {
    uint32_t cand[kWarpCand];           // candidate slots, groups back to back
    uint32_t hits[32][kGroupSlots];     // per home lane: hit bits of its group's candidates
};

// Static neighbours of one slot in the walk's order: list entries and sum.
template <bool kExact>
__device__ __forceinline__ float density_statics(const SceneDesc& sc, uint32_t i, const float4& p, const Walk& w,
                                                 const StaticTables& st, const NbrArgs& nl, uint64_t keep,
                                                 uint32_t& scnt)
{
    float sum_s = 0.f;
    scnt = 0;
    if (!w.near_static) return sum_s;
    const uint32_t stride = nl.stride;
    const float h = sc.h;
    walk_neighbours_cells<kExact, false>(
        sc, i, p, w, nullptr, nullptr, st, [](uint32_t, const float4&, float) {},
        [&](uint32_t e, const float4&, float r2) {
            if (scnt < kMaxSNbr) store_list(nl.snbr + (size_t)scnt * stride + i, e, keep);
            ++scnt;
            sum_s = __fadd_rn(sum_s, w0_of<kExact>(r2, h));
        },
        [](uint32_t) {});
    return sum_s;
}

// Step 2 for one group whose candidates fill kWords register slots: for each
// home, one ballot per slot (bit l of word s: candidate 32 s + l is within h).
template <bool kExact, uint32_t kWords>
__device__ __forceinline__ void group_ballots(uint32_t group, const float (&qx)[kGroupSlots],
                                              const float (&qy)[kGroupSlots], const float (&qz)[kGroupSlots],
                                              const float4& p, float h2, GroupSmem& sm, uint32_t wl)
{
    uint32_t hm = group;
    while (hm) {
        const int hl = __ffs(hm) - 1;
        hm &= hm - 1u;
        const float4 hp = make_float4(__shfl_sync(0xffffffffu, p.x, hl), __shfl_sync(0xffffffffu, p.y, hl),
                                      __shfl_sync(0xffffffffu, p.z, hl), 0.f);
        uint32_t b[kGroupSlots];
#pragma unroll
        for (uint32_t s = 0; s < kGroupSlots; ++s) {
            b[s] = 0u;
            if (s < kWords) {
                const float r2 = pair_r2<kExact>(make_float4(qx[s], qy[s], qz[s], 0.f), hp);
                b[s] = __ballot_sync(0xffffffffu, !(r2 > h2));
            }
        }
        if (wl == 0u) {
            uint4* d = reinterpret_cast<uint4*>(sm.hits[hl]);
            d[0] = make_uint4(b[0], b[1], b[2], b[3]);
            if (kWords > 4) d[1] = make_uint4(b[4], b[5], b[6], b[7]);
        }
    }
}

// `lane` = the slot's place in the tile; a warp's 32 lanes share one tile.
template <bool kExact>
__device__ __forceinline__ void density_group_tile(uint32_t tile_index, const Tile& tile, uint32_t lane,
                                                   const SceneDesc* scenes, const float4* __restrict__ pos,
                                                   float4* __restrict__ vel, const uint32_t* __restrict__ start,
                                                   const StaticTables& st, const NbrArgs& nl, GroupSmem& sm)
{
    constexpr unsigned kFull = 0xffffffffu;
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + lane;
    const bool valid = i < tile.end;
    if (__ballot_sync(kFull, valid) == 0u) return;
    const uint32_t wl = lane & 31u;
    const float h = sc.h, h2 = sc.h2;
    const float4 p = valid ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool nonfinite_seen = *nl.nonfinite != 0u;
    uint32_t code, ex[3], ey[3], ez[3];
    bool near_static;
    bool elig, dup;
    {
        const Neighbourhood nb = neighbourhood(p.x, p.y, p.z, h);
        elig = valid && finite3(p);
        dup = nb_span(nb) >= sc.buckets;          // the 27 buckets may repeat
        code = nb.ex1 + nb.ey1 + nb.ez1;
        ex[0] = nb.ex0; ex[1] = nb.ex1; ex[2] = nb.ex2;
        ey[0] = nb.ey0; ey[1] = nb.ey1; ey[2] = nb.ey2;
        ez[0] = nb.ez0; ez[1] = nb.ez1; ez[2] = nb.ez2;
        // a static particle lies in the cell's neighbourhood (its bit in the
        // static-presence bitmap)
        const uint32_t own = code & sc.sbm_mask;
        near_static = sc.s && ((__ldg(st.sbitmap + sc.sbm_off + (own >> 5)) >> (own & 31u)) & 1u);
    }
    const uint32_t near_mask = __ballot_sync(kFull, near_static);
    const uint32_t delta = sc.p_off - __ldg(start + sc.q_off);
    const uint32_t stride = nl.stride;
    const uint64_t keep = l2_policy_keep();
    const int ka = (int)wl / 9, kb = ((int)wl / 3) % 3, kc = (int)wl % 3;   // this lane's neighbour cell
    uint32_t pending = __ballot_sync(kFull, elig);
    uint32_t fallback = __ballot_sync(kFull, valid && !elig);
    uint32_t waiting = 0;       // homes whose hit bits wait in shared memory
    uint32_t cursor = 0;
    uint32_t my_base = 0, my_words = 0, my_self = 0;
    bool my_sdup = false;
    uint32_t cnt = 0;
    float sum_d = 0.f;

    // step 3 for this lane's home: its hits in candidate order appended to
    // its neighbour list and summed, one hit per iteration.  The hit words
    // sit in registers and shift down as each runs out, so a lane's loop runs
    // once per hit, not once per word and hit.  The home's own slot is one
    // known candidate where the buckets are distinct (my_self), else
    // compared at every hit.
    auto sum_hits = [&]() {
        const uint32_t* cw = sm.cand + my_base;
        const uint4 lo = reinterpret_cast<const uint4*>(sm.hits[wl])[0];
        const uint4 hi = reinterpret_cast<const uint4*>(sm.hits[wl])[1];
        uint32_t w0 = lo.x, w1 = lo.y, w2 = lo.z, w3 = lo.w, w4 = hi.x, w5 = hi.y, w6 = hi.z, w7 = hi.w;
        // words past the group's own hold another group's bits
        if (my_words < 2) w1 = 0u;
        if (my_words < 3) w2 = 0u;
        if (my_words < 4) w3 = 0u;
        if (my_words < 5) w4 = 0u;
        if (my_words < 6) w5 = 0u;
        if (my_words < 7) w6 = 0u;
        if (my_words < 8) w7 = 0u;
        const uint32_t self_word = dup ? ~0u : my_self >> 5, m = ~(1u << (my_self & 31u));
        w0 &= self_word == 0u ? m : ~0u; w1 &= self_word == 1u ? m : ~0u;
        w2 &= self_word == 2u ? m : ~0u; w3 &= self_word == 3u ? m : ~0u;
        w4 &= self_word == 4u ? m : ~0u; w5 &= self_word == 5u ? m : ~0u;
        w6 &= self_word == 6u ? m : ~0u; w7 &= self_word == 7u ? m : ~0u;
        uint32_t base = 0;
        for (;;) {
            while (w0 == 0u) {
                if ((w1 | w2 | w3 | w4 | w5 | w6 | w7) == 0u) return;
                w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6; w6 = w7; w7 = 0u;
                base += 32u;
            }
            const uint32_t b = (uint32_t)__ffs(w0) - 1u;
            w0 &= w0 - 1u;
            const uint32_t j = cw[base + b];
            if (dup && j == i) continue;
            if (cnt < kMaxNbr) store_list(nl.nbr + (size_t)cnt * stride + i, j, keep);
            ++cnt;
            sum_d = __fadd_rn(sum_d, w0_of<kExact>(pair_r2<kExact>(__ldg(pos + j), p), h));
        }
    };

    while (pending) {
        const int leader = __ffs(pending) - 1;
        const uint32_t lcode = __shfl_sync(kFull, code, leader);
        const uint32_t group = __ballot_sync(kFull, elig && code == lcode) & pending;
        pending &= ~group;
        // step 1: the group's 27 buckets, one per lane
        const uint32_t gx0 = __shfl_sync(kFull, ex[0], leader), gx1 = __shfl_sync(kFull, ex[1], leader),
                       gx2 = __shfl_sync(kFull, ex[2], leader);
        const uint32_t gy0 = __shfl_sync(kFull, ey[0], leader), gy1 = __shfl_sync(kFull, ey[1], leader),
                       gy2 = __shfl_sync(kFull, ey[2], leader);
        const uint32_t gz0 = __shfl_sync(kFull, ez[0], leader), gz1 = __shfl_sync(kFull, ez[1], leader),
                       gz2 = __shfl_sync(kFull, ez[2], leader);
        const uint32_t hsh = pick3(ka, gx0, gx1, gx2) + pick3(kb, gy0, gy1, gy2) + pick3(kc, gz0, gz1, gz2);
        // The reference's static buckets of the 27 cells (hash % s): where
        // two coincide its static walk visits that bucket twice, and so does
        // density_statics then (walking the reference's own table).
        bool sdup = false;
        if (group & near_mask) {
            const uint32_t sb = wl < 27u ? fast_mod(hsh, sc.fm_s) : ~wl;
            const unsigned peers = __match_any_sync(kFull, sb);       // every lane takes part
            sdup = __ballot_sync(kFull, wl < 27u && __popc(peers) > 1) != 0u;
        }
        uint32_t beg = 0, len = 0;
        if (wl < 27u) {
            const uint32_t bk = sc.q_off + fast_mod(hsh, sc.fm_b);
            beg = max(__ldg(start + bk) + delta, sc.p_off);
            const uint32_t end = min(__ldg(start + bk + 1) + delta, sc.p_off + sc.n);
            len = end > beg ? end - beg : 0u;
        }
        uint32_t incl = len;
#pragma unroll
        for (uint32_t o = 1; o < 32u; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, incl, o);
            if (wl >= o) incl += t;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        if (total > kGroupSlots * 32u) {          // a crowded cell: the per-slot walk
            fallback |= group;
            continue;
        }
        if (cursor + total > kWarpCand) {        // shared memory full: finish the waiting homes
            if ((waiting >> wl) & 1u) sum_hits();
            waiting = 0;
            cursor = 0;
            __syncwarp();
        }
        uint32_t* cw = sm.cand + cursor;
        const uint32_t excl = incl - len;
        for (uint32_t m = 0; m < len; ++m) cw[excl + m] = beg + m;
        __syncwarp();
        const uint32_t words = (total + 31u) >> 5;
        float qx[kGroupSlots], qy[kGroupSlots], qz[kGroupSlots];
#pragma unroll
        for (uint32_t s = 0; s < kGroupSlots; ++s) {
            const uint32_t c = s * 32u + wl;
            qx[s] = qy[s] = qz[s] = __int_as_float(0x7f800000);   // +inf: never within h of a finite home
            if (c < total) {
                const float4 q = __ldg(pos + cw[c]);
                qx[s] = q.x; qy[s] = q.y; qz[s] = q.z;
            }
        }
        // the home's own slot: its place among the candidates of the centre bucket (k = 13)
        const uint32_t beg13 = __shfl_sync(kFull, beg, 13), pre13 = __shfl_sync(kFull, excl, 13);
        // step 2: one ballot per home and register slot (a straight-line
        // instance per slot count)
        switch (words) {
        case 1: group_ballots<kExact, 1>(group, qx, qy, qz, p, h2, sm, wl); break;
        case 2: group_ballots<kExact, 2>(group, qx, qy, qz, p, h2, sm, wl); break;
        case 3: group_ballots<kExact, 3>(group, qx, qy, qz, p, h2, sm, wl); break;
        case 4: group_ballots<kExact, 4>(group, qx, qy, qz, p, h2, sm, wl); break;
        case 5: group_ballots<kExact, 5>(group, qx, qy, qz, p, h2, sm, wl); break;
        case 6: group_ballots<kExact, 6>(group, qx, qy, qz, p, h2, sm, wl); break;
        case 7: group_ballots<kExact, 7>(group, qx, qy, qz, p, h2, sm, wl); break;
        default: group_ballots<kExact, 8>(group, qx, qy, qz, p, h2, sm, wl); break;
        }
        if ((group >> wl) & 1u) {
            my_base = cursor;
            my_words = words;
            my_self = pre13 + (i - beg13);
            my_sdup = sdup;
        }
        waiting |= group;
        cursor += total;
        __syncwarp();
    }
    if ((waiting >> wl) & 1u) sum_hits();
    if ((fallback >> wl) & 1u) {
        density_tile<kExact>(tile_index, tile, lane, scenes, pos, vel, start, st, nl);
        return;
    }
    if (!elig) return;
    // statics, walked per slot where the cell's neighbourhood holds any (its
    // bit in the static-presence bitmap); the reference's own table only
    // where the group's reference buckets repeat
    uint32_t scnt = 0;
    float sum_s = 0.f;
    if (near_static) {
        Walk w = make_walk<kExact>(sc, p, st.sbitmap, nonfinite_seen);
        w.ref_walk = my_sdup;
        sum_s = density_statics<kExact>(sc, i, p, w, st, nl, keep, scnt);
    }
    const bool overflow = cnt > kMaxNbr || scnt > kMaxSNbr;
    if (overflow) atomicOr(nl.tile_overflow + tile_index, 1u);   // cleared by the overflow force pass
    nl.ncount[i] = overflow ? (kOverflow | (kOverflow << 16)) : (cnt | (scnt << 16));
    // SF:497-498
    const float rho = __fadd_rn(sc.self_density,
                                __fmul_rn(__fadd_rn(__fmul_rn(sum_d, sc.mass), __fmul_rn(sum_s, sc.mass)), sc.kc));
    const float pressure = __fmul_rn(sc.gas, __fsub_rn(rho, sc.rho0));
    reinterpret_cast<float*>(vel + i)[3] = pressure;
}

// Marks, for every static particle, the bitmap bits of the 27 cells whose
// neighbourhood holds its cell.
__device__ __forceinline__ void static_bitmap_tile(const Tile& tile, const SceneDesc* scenes, const float4* spos,
                                                   uint32_t* sbitmap)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    if (i >= tile.end) return;
    const float4 q = spos[i];
    const Neighbourhood nb = neighbourhood(q.x, q.y, q.z, sc.h);
    for (int k = 0; k < 27; ++k) {
        const uint32_t code = neighbour_hash(nb, k / 9, (k / 3) % 3, k % 3) & sc.sbm_mask;
        atomicOr(sbitmap + sc.sbm_off + (code >> 5), 1u << (code & 31u));
    }
}

// ---- stage: force + integrate + rehash -------------------------------------
//
// UpdateParticleDynamics (SF:503-656): pressure force dir (p_i + p_j) W1 and
// viscosity (v_j - v_i) W2 over dynamic neighbours; dir |p_i| W1 over static
// neighbours (their viscosity term is multiplied by 0 in the reference,
// SF:629, and is omitted); scale by m / (2 rho_i) C and mu m C; add triangle
// forces; a = F / rho_i + g; semi-implicit Euler; new key; count.
//
// The neighbours come from the density pass's list, in the same order as the
// buckets were walked.  Particles whose list overflowed are left to
// force_overflow_tile, which walks their buckets.

struct PairSums {
    float3 fp, fv, fs;
};

// Coincident pair: the reference's RandomDirection((float)threadID), its
// thread being the particle's buffer index (SF:576-580, 610-614).  The fast
// form seeds with the input index instead, which keeps the tag array out of
// the force loop's registers.
template <bool kExact>
__device__ __forceinline__ float3 coincident_direction(const float4& p, const uint32_t* tag, uint32_t i)
{
    return random_direction((float)(kExact ? __ldg(tag + i) : __float_as_uint(p.w)));
}

// One dynamic neighbour: pressure force dir (p_i + p_j) W1 and viscosity
// (v_j - v_i) W2 (SF:567-589).  Pairs at r >= h add nothing in the
// reference (the kernels return 0) and are skipped.  kExact follows the
// reference's operations one for one: dir / r by true division, each
// product rounded, no fused multiply-adds.
// kDefer: a coincident pair adds nothing and sets *coincident instead (the
// caller then repeats the sums with kDefer = false, in the same order).
template <bool kExact, bool kDefer = false>
__device__ __forceinline__ void add_dynamic_pair(PairSums& s, const float4& p, const float4& v, float pi, float h,
                                                 const float4& q, const float4& u, const uint32_t* tag, uint32_t i,
                                                 bool* coincident = nullptr)
{
    float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
    const float r2 = kExact ? __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz))
                            : __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    const float rinv = kExact ? 0.f : rsqrtf(r2);
    const float r = root_of<kExact>(r2, rinv);
    if (r >= h) return;          // a NaN distance is kept (SF:126-139)
    if (r2 == 0.f || r == 0.f) {
        if (kDefer) {
            *coincident = true;
            return;
        }
        const float3 d = coincident_direction<kExact>(p, tag, i);
        dx = d.x; dy = d.y; dz = d.z;
    } else if (kExact) {
        dx = __fdiv_rn(dx, r); dy = __fdiv_rn(dy, r); dz = __fdiv_rn(dz, r);
    } else {
        dx = __fmul_rn(dx, rinv); dy = __fmul_rn(dy, rinv); dz = __fmul_rn(dz, rinv);
    }
    const float w = __fsub_rn(h, r);
    const float w1 = __fmul_rn(__fmul_rn(-3.f, w), w);
    const float w2 = __fmul_rn(6.f, w);
    const float pij = __fadd_rn(pi, u.w);
    if (kExact) {
        s.fp.x = __fadd_rn(s.fp.x, __fmul_rn(__fmul_rn(dx, pij), w1));
        s.fp.y = __fadd_rn(s.fp.y, __fmul_rn(__fmul_rn(dy, pij), w1));
        s.fp.z = __fadd_rn(s.fp.z, __fmul_rn(__fmul_rn(dz, pij), w1));
        s.fv.x = __fadd_rn(s.fv.x, __fmul_rn(__fsub_rn(u.x, v.x), w2));
        s.fv.y = __fadd_rn(s.fv.y, __fmul_rn(__fsub_rn(u.y, v.y), w2));
        s.fv.z = __fadd_rn(s.fv.z, __fmul_rn(__fsub_rn(u.z, v.z), w2));
    } else {
        const float pp = __fmul_rn(pij, w1);
        s.fp.x = __fmaf_rn(dx, pp, s.fp.x);
        s.fp.y = __fmaf_rn(dy, pp, s.fp.y);
        s.fp.z = __fmaf_rn(dz, pp, s.fp.z);
        s.fv.x = __fmaf_rn(__fsub_rn(u.x, v.x), w2, s.fv.x);
        s.fv.y = __fmaf_rn(__fsub_rn(u.y, v.y), w2, s.fv.y);
        s.fv.z = __fmaf_rn(__fsub_rn(u.z, v.z), w2, s.fv.z);
    }
}

// One static neighbour: dir |p_i| W1 (SF:600-622).  The reference also sums a
// static viscosity term and multiplies it by 0 (SF:629): for finite values
// that adds a signed zero to a force that is never -0, so it is omitted.
template <bool kExact, bool kDefer = false>
__device__ __forceinline__ void add_static_pair(PairSums& s, const float4& p, float api, float h, const float4& q,
                                                const uint32_t* tag, uint32_t i, bool* coincident = nullptr)
{
    float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
    const float r2 = kExact ? __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz))
                            : __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    const float rinv = kExact ? 0.f : rsqrtf(r2);
    const float r = root_of<kExact>(r2, rinv);
    if (r >= h) return;          // a NaN distance is kept (SF:126-139)
    if (r2 == 0.f || r == 0.f) {
        if (kDefer) {
            *coincident = true;
            return;
        }
        const float3 d = coincident_direction<kExact>(p, tag, i);
        dx = d.x; dy = d.y; dz = d.z;
    } else if (kExact) {
        dx = __fdiv_rn(dx, r); dy = __fdiv_rn(dy, r); dz = __fdiv_rn(dz, r);
    } else {
        dx = __fmul_rn(dx, rinv); dy = __fmul_rn(dy, rinv); dz = __fmul_rn(dz, rinv);
    }
    const float w = __fsub_rn(h, r);
    const float w1 = __fmul_rn(__fmul_rn(-3.f, w), w);
    if (kExact) {
        s.fs.x = __fadd_rn(s.fs.x, __fmul_rn(__fmul_rn(dx, api), w1));
        s.fs.y = __fadd_rn(s.fs.y, __fmul_rn(__fmul_rn(dy, api), w1));
        s.fs.z = __fadd_rn(s.fs.z, __fmul_rn(__fmul_rn(dz, api), w1));
    } else {
        const float pp = __fmul_rn(api, w1);
        s.fs.x = __fmaf_rn(dx, pp, s.fs.x);
        s.fs.y = __fmaf_rn(dy, pp, s.fs.y);
        s.fs.z = __fmaf_rn(dz, pp, s.fs.z);
    }
}

// SF:626-645: scale the sums, add triangle forces and gravity, integrate,
// store the moved particle and its new key.  The reference starts the total
// from a zero vector (SF:631-635); kExact keeps that first add.
// The boundary mesh and its triangle cells.
struct TriangleMesh {
    const float* tris;          // 9 floats per triangle
    const uint32_t* cells;
    const uint32_t* list;
};

// SF:636-637: the force of every triangle, added in triangle order.  With
// triangle cells only the triangles listed for the particle's cell are
// evaluated, still in increasing index: every other one lies beyond
// kTriangleReach and adds the zero vector, which leaves the total as it is
// (the total is never -0, as it starts from +0).  A point outside the cells
// (or NaN) is beyond reach of every triangle.
__device__ __forceinline__ void add_triangle_forces(const SceneDesc& sc, const TriangleMesh& tm, float3 p, float3& f)
{
    if (!sc.t) return;
    auto add = [&](uint32_t t) {
        const float3 tf = triangle_force(p, tm.tris + 9u * t);
        f.x = __fadd_rn(f.x, tf.x); f.y = __fadd_rn(f.y, tf.y); f.z = __fadd_rn(f.z, tf.z);
    };
    // no grid, or a non-finite particle: every triangle, as the reference
    // evaluates them (each returns NaN for a NaN distance, SF:219-220)
    if (sc.tg_nx == 0 || !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) {
        for (uint32_t t = 0; t < sc.t; ++t) add(sc.t_off + t);
        return;
    }
    const float cx = floorf(__fmul_rn(__fsub_rn(p.x, sc.tg_ox), sc.tg_inv));
    const float cy = floorf(__fmul_rn(__fsub_rn(p.y, sc.tg_oy), sc.tg_inv));
    const float cz = floorf(__fmul_rn(__fsub_rn(p.z, sc.tg_oz), sc.tg_inv));
    if (!(cx >= 0.f && cx < (float)sc.tg_nx && cy >= 0.f && cy < (float)sc.tg_ny && cz >= 0.f &&
          cz < (float)sc.tg_nz))
        return;
    const uint32_t c = sc.tg_cell_off + ((uint32_t)cz * sc.tg_ny + (uint32_t)cy) * sc.tg_nx + (uint32_t)cx;
    const uint32_t end = __ldg(tm.cells + c + 1);
    for (uint32_t k = __ldg(tm.cells + c); k < end; ++k) add(__ldg(tm.list + k));
}

template <bool kRecordAccel, bool kExact>
__device__ __forceinline__ uint32_t integrate_particle(const SceneDesc& sc, uint32_t i, const float4& p, const float4& v,
                                                       float rho, const PairSums& s, const TriangleMesh& tm,
                                                       float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                       uint32_t* __restrict__ key_out, float4* accel,
                                                       uint32_t* nonfinite_next)
{
    const float s1 = __fmul_rn(__fdiv_rn(sc.mass, __fmul_rn(2.f, rho)), sc.kc);
    const float s2 = __fmul_rn(__fmul_rn(sc.visc, sc.mass), sc.kc);
    float3 f;
    const float z = 0.f;
    f.x = kExact ? __fadd_rn(z, __fmul_rn(s.fp.x, s1)) : __fmul_rn(s.fp.x, s1);
    f.y = kExact ? __fadd_rn(z, __fmul_rn(s.fp.y, s1)) : __fmul_rn(s.fp.y, s1);
    f.z = kExact ? __fadd_rn(z, __fmul_rn(s.fp.z, s1)) : __fmul_rn(s.fp.z, s1);
    f.x = __fadd_rn(__fadd_rn(f.x, __fmul_rn(s.fv.x, s2)), __fmul_rn(s.fs.x, s1));
    f.y = __fadd_rn(__fadd_rn(f.y, __fmul_rn(s.fv.y, s2)), __fmul_rn(s.fs.y, s1));
    f.z = __fadd_rn(__fadd_rn(f.z, __fmul_rn(s.fv.z, s2)), __fmul_rn(s.fs.z, s1));
    add_triangle_forces(sc, tm, make_float3(p.x, p.y, p.z), f);
    float3 acc;
    acc.x = __fadd_rn(__fdiv_rn(f.x, rho), sc.gx);
    acc.y = __fadd_rn(__fdiv_rn(f.y, rho), sc.gy);
    acc.z = __fadd_rn(__fdiv_rn(f.z, rho), sc.gz);
    float3 nv, np;
    nv.x = __fadd_rn(v.x, __fmul_rn(acc.x, sc.dt));
    nv.y = __fadd_rn(v.y, __fmul_rn(acc.y, sc.dt));
    nv.z = __fadd_rn(v.z, __fmul_rn(acc.z, sc.dt));
    np.x = __fadd_rn(p.x, __fmul_rn(nv.x, sc.dt));
    np.y = __fadd_rn(p.y, __fmul_rn(nv.y, sc.dt));
    np.z = __fadd_rn(p.z, __fmul_rn(nv.z, sc.dt));
    const uint32_t k = fast_mod(cell_hash(np.x, np.y, np.z, sc.h), sc.fm_b);
    if (!(isfinite(np.x) && isfinite(np.y) && isfinite(np.z))) atomicOr(nonfinite_next, 1u);
    pos_out[i] = make_float4(np.x, np.y, np.z, p.w);
    vel_out[i] = make_float4(nv.x, nv.y, nv.z, v.w);
    key_out[i] = k;
    if (kRecordAccel) accel[i] = make_float4(acc.x, acc.y, acc.z, 0.f);
    return k;
}

// The neighbour lists are dead once the force pass has read them: the next
// density pass rewrites every entry a force pass reads.  So each warp drops
// its rows' lines from L2 without writing them back (PTX discard.global.L2:
// the line's contents become undefined), which keeps the density pass's list
// writes out of DRAM while they are still in L2.  Only where the warp's 32
// slots fill their lines alone: every lane a slot of this tile, the first
// slot a multiple of 32 (rows start at multiples of 32 entries, list_stride).
// `rows` / `srows`: this lane's dynamic / static entries read (0 if none).
__device__ __forceinline__ void discard_read_lists(const Tile& tile, uint32_t i, uint32_t lane, const NbrArgs& nl,
                                                   uint32_t rows, uint32_t srows)
{
    const uint32_t wl = lane & 31u;
    const uint32_t ws = i - wl;                        // the warp's first slot
    const bool whole = __ballot_sync(0xffffffffu, i < tile.end) == 0xffffffffu && (ws & 31u) == 0u &&
                       (nl.stride & 31u) == 0u;
    const uint32_t dr = __reduce_max_sync(0xffffffffu, rows);
    const uint32_t sr = __reduce_max_sync(0xffffffffu, srows);
    if (!whole) return;
    for (uint32_t k = wl; k < dr; k += 32u)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(nl.nbr + (size_t)k * nl.stride + ws) : "memory");
    for (uint32_t k = wl; k < sr; k += 32u)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(nl.snbr + (size_t)k * nl.stride + ws) : "memory");
}

// Where the force pass writes and counts.
struct ForceOut {
    float4* pos_out;
    float4* vel_out;
    uint32_t* key_out;
    uint32_t* arrival;
    uint32_t* count;
    float4* accel;
    uint32_t* nonfinite_next;   // set when a new position is not finite
};

// `lane` = the slot's place in the tile (threadIdx.x when a CTA covers one
// tile; CTAs of other sizes pass theirs).
template <bool kRecordAccel, bool kExact>
__device__ __forceinline__ void force_tile(const Tile& tile, const SceneDesc* scenes, const float4* __restrict__ pos,
                                           const float4* __restrict__ vel, const uint32_t* __restrict__ tag,
                                           const StaticTables& st, const TriangleMesh& tm, const NbrArgs& nl,
                                           const ForceOut& o, uint32_t lane = threadIdx.x)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + lane;
    bool valid = i < tile.end;
    uint32_t g = 0;
    uint32_t listed = 0, slisted = 0;              // list entries this slot reads
    if (valid) {
        const uint32_t c = nl.ncount[i];
        const uint32_t cd = c & 0xFFFFu, cs = c >> 16;
        if (cd == kOverflow || cs == kOverflow) {
            valid = false;                         // handled by force_overflow_tile
        } else {
            listed = cd;
            slisted = cs;
            const float h = sc.h;
            const float4 p = pos[i];
            const float4 v = vel[i];
            const float pi = v.w;
            const float rho = __fadd_rn(__fdiv_rn(pi, sc.gas), sc.rho0);   // SF:541
            const uint32_t stride = nl.stride;
            // The sums over the lists.  Four neighbours per round: eight
            // position/velocity loads in flight.  The list entries of round
            // r + 1 are loaded while round r's neighbours arrive, so a round
            // waits on one load, not two.
            const uint64_t drop = l2_policy_drop();
            const float api = fabsf(pi);
            bool coincident = false;
            auto sums = [&](auto defer_tag) -> PairSums {
                constexpr bool kDefer = decltype(defer_tag)::value;
                PairSums s;
                s.fp = s.fv = s.fs = make_float3(0.f, 0.f, 0.f);
                const uint32_t* lp = nl.nbr + i;
                uint32_t k = 0;
                uint32_t n0 = 0, n1 = 0, n2 = 0, n3 = 0;
                if (SPH_NBR_BATCH == 4 && k + 4 <= cd) {
                    n0 = load_list(lp, drop); n1 = load_list(lp + stride, drop);
                    n2 = load_list(lp + 2 * (size_t)stride, drop); n3 = load_list(lp + 3 * (size_t)stride, drop);
                }
                for (; SPH_NBR_BATCH == 4 && k + 4 <= cd; k += 4, lp += 4 * (size_t)stride) {
                    const uint32_t j0 = n0, j1 = n1, j2 = n2, j3 = n3;
                    if (k + 8 <= cd) {
                        const uint32_t* ln = lp + 4 * (size_t)stride;
                        n0 = load_list(ln, drop); n1 = load_list(ln + stride, drop);
                        n2 = load_list(ln + 2 * (size_t)stride, drop); n3 = load_list(ln + 3 * (size_t)stride, drop);
                    }
                    const float4 q0 = __ldg(pos + j0), q1 = __ldg(pos + j1), q2 = __ldg(pos + j2), q3 = __ldg(pos + j3);
                    const float4 u0 = __ldg(vel + j0), u1 = __ldg(vel + j1), u2 = __ldg(vel + j2), u3 = __ldg(vel + j3);
                    add_dynamic_pair<kExact, kDefer>(s, p, v, pi, h, q0, u0, tag, i, &coincident);
                    add_dynamic_pair<kExact, kDefer>(s, p, v, pi, h, q1, u1, tag, i, &coincident);
                    add_dynamic_pair<kExact, kDefer>(s, p, v, pi, h, q2, u2, tag, i, &coincident);
                    add_dynamic_pair<kExact, kDefer>(s, p, v, pi, h, q3, u3, tag, i, &coincident);
                }
                for (; k < cd; ++k, lp += stride) {
                    const uint32_t j = load_list(lp, drop);
                    add_dynamic_pair<kExact, kDefer>(s, p, v, pi, h, __ldg(pos + j), __ldg(vel + j), tag, i, &coincident);
                }
                lp = nl.snbr + i;
                for (uint32_t k = 0; k < cs; ++k, lp += stride)
                    add_static_pair<kExact, kDefer>(s, p, api, h, static_entry_pos(load_list(lp, drop), st), tag, i,
                                                    &coincident);
                return s;
            };
            // Coincident pairs (r = 0, the reference's random direction) are
            // rare: the first pass leaves them out, and only a particle that
            // has one sums again with them, in the same order.  Keeping the
            // random-direction call out of the common loop made force 6 %
            // faster (0.160 against 0.171 ms on the 1M dam break).
            PairSums s = sums(std::integral_constant<bool, true>());
            if (coincident) s = sums(std::integral_constant<bool, false>());
            g = sc.q_off + integrate_particle<kRecordAccel, kExact>(sc, i, p, v, rho, s, tm, o.pos_out, o.vel_out,
                                                                    o.key_out, o.accel, o.nonfinite_next);
        }
    }
    discard_read_lists(tile, i, lane, nl, valid ? listed : 0u, valid ? slisted : 0u);
    const uint32_t r = warp_aggregated_increment(o.count, g, valid);
    if (valid) o.arrival[i] = r;
}

// Overflow particles: the same sums, walking the 27 cells directly.
template <bool kRecordAccel, bool kExact>
__device__ __forceinline__ void force_overflow_tile(const Tile& tile, const SceneDesc* scenes,
                                                    const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                    const uint32_t* __restrict__ tag, const uint32_t* __restrict__ start,
                                                    const StaticTables& st, const TriangleMesh& tm,
                                                    const NbrArgs& nl, const ForceOut& o)
{
    const SceneDesc& sc = scenes[tile.scene];
    const uint32_t i = tile.begin + threadIdx.x;
    bool valid = false;
    uint32_t g = 0;
    if (i < tile.end) {
        const uint32_t c = nl.ncount[i];
        valid = (c & 0xFFFFu) == kOverflow || (c >> 16) == kOverflow;
    }
    if (valid) {
        const float h = sc.h;
        const float4 p = pos[i];
        const float4 v = vel[i];
        const float pi = v.w;
        const float api = fabsf(pi);
        const float rho = __fadd_rn(__fdiv_rn(pi, sc.gas), sc.rho0);
        const Walk w = make_walk<kExact>(sc, p, st.sbitmap, *nl.nonfinite != 0u);
        PairSums s;
        s.fp = s.fv = s.fs = make_float3(0.f, 0.f, 0.f);
        walk_neighbours<kExact>(
            sc, i, p, w, pos, start, st,
            [&](uint32_t j, const float4& q, float) { add_dynamic_pair<kExact>(s, p, v, pi, h, q, __ldg(vel + j), tag, i); },
            [&](uint32_t, const float4& q, float) { add_static_pair<kExact>(s, p, api, h, q, tag, i); });
        g = sc.q_off + integrate_particle<kRecordAccel, kExact>(sc, i, p, v, rho, s, tm, o.pos_out, o.vel_out,
                                                                o.key_out, o.accel, o.nonfinite_next);
    }
    const uint32_t r = warp_aggregated_increment(o.count, g, valid);
    if (valid) o.arrival[i] = r;
}

// ---- views of the step arguments ------------------------------------------

__device__ __forceinline__ NbrArgs nbr_args(const StepArgs& a)
{
    return NbrArgs{a.nbr, a.snbr, a.ncount, a.tile_overflow, a.nbr_stride, a.nonfinite};
}

__device__ __forceinline__ StaticTables static_tables(const StepArgs& a)
{
    return StaticTables{a.spos, a.sstart, a.spos_ref, a.sstart_ref, a.sbitmap};
}

__device__ __forceinline__ TriangleMesh triangle_mesh(const StepArgs& a)
{
    return TriangleMesh{a.tris, a.tri_cells, a.tri_list};
}

__device__ __forceinline__ ForceOut force_out(const StepArgs& a)
{
    return ForceOut{a.pos_tmp, a.vel_tmp, a.key, a.arrival, a.count, a.accel, a.nonfinite + 1};
}

}  // namespace sph
