// sph_shapes.cu -- launch shapes of the two neighbour passes, for the
// autotuner.
//
// The default step launches the density and force passes with one CTA of
// kTileThreads threads per tile and a register bound of 7 resident CTAs per
// SM.  Here the same routines (density_group_tile, force_tile, default
// arithmetic) run under other shapes: CTAs of 64 or 256 threads (half a tile,
// or two tiles) and other register bounds.  Density shape 5 runs the per-slot
// walk (density_tile) instead of the group walk.  Each shape does the same
// work slot for slot, so results are bit-identical across shapes; only the
// time differs.  The reference sizes its OpenCL work groups from device queries
// (SimulationEngineGPUKernels.cpp:260-291); this engine measures instead
// (sph_batch_autotune, sph_engine_autotune).
#include "sph_state.h"

namespace sph {

// slot -> (tile, place in the tile) for a CTA of kThreads threads
template <int kThreads>
__device__ __forceinline__ bool shaped_slot(const StepArgs& a, uint32_t* tile, uint32_t* lane)
{
    const uint32_t g = blockIdx.x * (uint32_t)kThreads + threadIdx.x;
    *tile = g / (uint32_t)kTileThreads;
    *lane = g % (uint32_t)kTileThreads;
    return *tile < a.num_tiles;
}

template <int kThreads, int kMinCtas, bool kSlotWalk = false>
__global__ void __launch_bounds__(kThreads, kMinCtas) k_density_shaped(StepArgs a)
{
    __shared__ __align__(16) GroupSmem gsm[kSlotWalk ? 1 : kThreads / 32];
    uint32_t t, lane;
    if (!shaped_slot<kThreads>(a, &t, &lane)) return;        // whole warps
    if (kSlotWalk)
        density_tile<false>(t, a.tiles[t], lane, a.scenes, a.pos, a.vel, a.start, static_tables(a), nbr_args(a));
    else
        density_group_tile<false>(t, a.tiles[t], lane, a.scenes, a.pos, a.vel, a.start, static_tables(a),
                                  nbr_args(a), gsm[threadIdx.x >> 5]);
}

template <int kThreads, int kMinCtas>
__global__ void __launch_bounds__(kThreads, kMinCtas) k_force_shaped(StepArgs a)
{
    uint32_t t, lane;
    if (!shaped_slot<kThreads>(a, &t, &lane)) return;        // whole warps
    force_tile<false, false>(a.tiles[t], a.scenes, a.pos, a.vel, a.tag, static_tables(a), triangle_mesh(a),
                             nbr_args(a), force_out(a), lane);
}

template <int kThreads, int kMinCtas, bool kSlotWalk = false>
static cudaError_t launch_pair(bool density, const StepArgs& a, cudaStream_t s)
{
    const uint32_t slots = a.num_tiles * (uint32_t)kTileThreads;
    const unsigned grid = (slots + kThreads - 1) / kThreads;
    if (density)
        k_density_shaped<kThreads, kMinCtas, kSlotWalk><<<grid, kThreads, 0, s>>>(a);
    else
        k_force_shaped<kThreads, kMinCtas><<<grid, kThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_shaped(int shape, bool density, const StepArgs& a, cudaStream_t s)
{
    switch (shape) {
    case 1: return launch_pair<64, 14>(density, a, s);
    case 2: return launch_pair<256, 3>(density, a, s);
    case 3: return launch_pair<128, 6>(density, a, s);
    case 4: return launch_pair<128, 8>(density, a, s);
    case 5:     // density only: the per-slot walk (density_tile)
        return density ? launch_pair<kTileThreads, SPH_DENSITY_MIN_CTAS, true>(true, a, s) : cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;     // shape 0 is the default kernel
    }
}

}  // namespace sph
