// sph_noalloc.cu -- the counting sort for callers that cannot allocate.
//
// Some callers cannot call cudaMalloc: code running under a caller-owned
// memory pool or allocator that forbids driver allocations, code inside a
// simulation loop that must not trigger allocation (and its implicit
// synchronisation) mid-frame, or plugins whose host application owns all
// device memory.  sph_cell_sort_noalloc serves them: the caller passes device
// buffers for the inputs and outputs, and the sort's scratch (bucket
// counters, arrival ranks, the slot permutation, the scan's tile status) lives
// in one file-scope __device__ array of fixed size, so the call allocates
// nothing.
//
// That array is a fixed cost: every GPU that loads this library holds it
// (about 4.2 MiB) until the process exits.  All calls share it and it keeps
// the last call's contents, so each call clears the parts that must start at
// zero; calls that overlap on the GPU (different streams, or different host
// threads on one device) race on it and must be serialised by the caller.
#include <cuda.h>

#include <mutex>

#include "sph_state.h"

namespace sph {
namespace {

constexpr uint32_t kNoAllocMaxParticles = 1u << 18;   // SPH_NOALLOC_MAX_PARTICLES
constexpr uint32_t kNoAllocMaxBuckets = 1u << 19;     // SPH_NOALLOC_MAX_BUCKETS
constexpr uint32_t kNoAllocMaxScanTiles = (kNoAllocMaxBuckets + 1 + kScanTile - 1) / kScanTile;

// Scratch layout (32-bit words): count[max_buckets + 1] | arrival[max_n] |
// perm[max_n] | ticket | error | pad to 8 bytes | scan status (64-bit words).
constexpr size_t kCountWords = kNoAllocMaxBuckets + 4;   // rounded up to a multiple of 4
constexpr size_t kArrivalOff = kCountWords;
constexpr size_t kPermOff = kArrivalOff + kNoAllocMaxParticles;
constexpr size_t kTicketOff = kPermOff + kNoAllocMaxParticles;
constexpr size_t kErrOff = kTicketOff + 1;
constexpr size_t kStatusOff = kErrOff + 3;                // 8-byte aligned (kErrOff + 3 is even)
constexpr size_t kScratchWords = kStatusOff + 2 * (size_t)kNoAllocMaxScanTiles;
static_assert(kStatusOff % 2 == 0, "scan status must be 8-byte aligned");

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

struct NoAllocArgs {
    const float* pos;      // n x 3, device
    uint32_t n;
    float h;
    FastMod fm;
    uint32_t buckets;
    uint32_t* keys;        // n, device
    uint32_t* starts;      // buckets + 1, device
    uint32_t* order;       // n, device
    uint32_t* scratch;     // device address of g_noalloc_scratch
};

// Zero the counters this call scans, the scan's tile status, ticket and
// error word: all keep the previous call's values otherwise.
__global__ void __launch_bounds__(kTileThreads) k_na_clear(NoAllocArgs a, uint32_t scan_tiles)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t <= a.buckets; t += stride) a.scratch[t] = 0u;
    unsigned long long* status = reinterpret_cast<unsigned long long*>(a.scratch + kStatusOff);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < scan_tiles; t += stride) status[t] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.scratch[kTicketOff] = 0u;
        a.scratch[kErrOff] = 0u;
    }
}

// key = GetHash(GetCell(p)) % buckets and a warp-aggregated count, as
// hash_count_tile does for the engine (SF:321-331).
__global__ void __launch_bounds__(kTileThreads) k_na_hash_count(NoAllocArgs a)
{
    const uint32_t i = blockIdx.x * kTileThreads + threadIdx.x;
    const bool valid = i < a.n;
    uint32_t k = 0;
    if (valid) {
        const float x = a.pos[3ull * i], y = a.pos[3ull * i + 1], z = a.pos[3ull * i + 2];
        k = fast_mod(cell_hash(x, y, z, a.h), a.fm);
    }
    const uint32_t r = warp_aggregated_increment(a.scratch, k, valid);
    if (valid) {
        a.keys[i] = k;
        a.scratch[kArrivalOff + i] = r;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_na_scan(NoAllocArgs a)
{
    __shared__ ScanSmem sm;
    if (threadIdx.x == 0) sm.tile = atomicAdd(a.scratch + kTicketOff, 1u);
    __syncthreads();
    scan_tile(sm.tile, a.scratch, a.starts, a.buckets + 1u,
              reinterpret_cast<unsigned long long*>(a.scratch + kStatusOff), a.scratch + kErrOff, sm);
}

__global__ void __launch_bounds__(kTileThreads) k_na_scatter(NoAllocArgs a)
{
    const uint32_t i = blockIdx.x * kTileThreads + threadIdx.x;
    if (i >= a.n) return;
    const uint32_t slot = a.starts[a.keys[i]] + a.scratch[kArrivalOff + i];
    if (slot >= a.n) { atomicOr(a.scratch + kErrOff, DEV_ERR_SLOT_RANGE); return; }
    a.scratch[kPermOff + slot] = i;
}

// Deterministic placement: particle j goes to its bucket's start plus the
// number of the bucket's members with a larger input index, the order in
// which the reference's counting sort fills a bucket (gather_tile's rule).
__global__ void __launch_bounds__(kTileThreads) k_na_order(NoAllocArgs a)
{
    const uint32_t j = blockIdx.x * kTileThreads + threadIdx.x;
    if (j >= a.n) return;
    const uint32_t k = a.keys[j];
    const uint32_t b0 = a.starts[k], e0 = a.starts[k + 1];
    if (e0 < b0 || e0 > a.n) { atomicOr(a.scratch + kErrOff, DEV_ERR_BUCKET_RANGE); return; }
    const uint32_t* perm = a.scratch + kPermOff;
    uint32_t rank = 0;
    if (e0 - b0 <= kStableRankLimit) {
        for (uint32_t t = b0; t < e0; ++t) rank += perm[t] > j ? 1u : 0u;
    } else {
        rank = a.scratch[kArrivalOff + j];
    }
    a.order[b0 + rank] = j;
}

std::mutex g_symbol_mutex;

// The scratch array's device address, cached per device ordinal together
// with the id of the context it was looked up in.  cudaDeviceReset destroys
// the device's primary context and the module holding the array; the next
// runtime call creates a new context with a new id, whose array may sit at
// another address.  Context ids (cuCtxGetId) are never reused within a
// process, so a changed id means the cached address is stale.
struct ScratchSlot {
    unsigned long long ctx_id;
    uint32_t* ptr;
};
ScratchSlot g_symbol_slot[64] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Id of the current context (0 when there is none yet).  The two driver
// functions are resolved through the runtime, so the library does not link
// against the driver library directly.
sph_status current_context_id(unsigned long long* id)
{
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1{}, q2{};
        const cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        const cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || !f1 || !f2) {
            set_last_error("sph_cell_sort_noalloc: the driver's cuCtxGetCurrent / cuCtxGetId are unavailable");
            return SPH_ERR_CUDA;
        }
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) {
        set_last_error("sph_cell_sort_noalloc: cuCtxGetCurrent failed");
        return SPH_ERR_CUDA;
    }
    *id = 0;
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) {
        set_last_error("sph_cell_sort_noalloc: cuCtxGetId failed");
        return SPH_ERR_CUDA;
    }
    return SPH_OK;
}

// Device address of the scratch array on the current device.  It is looked
// up with cudaGetSymbolAddress, with the device current, on the first call
// on each device and again whenever the device's context has changed since
// (after a cudaDeviceReset).
sph_status scratch_address(int device, uint32_t** out)
{
    if (device < 0 || device >= 64) {
        set_last_error("device ordinal out of range");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_symbol_mutex);
    unsigned long long ctx_id = 0;
    sph_status st = current_context_id(&ctx_id);
    if (st != SPH_OK) return st;
    ScratchSlot& slot = g_symbol_slot[device];
    if (!slot.ptr || ctx_id == 0 || slot.ctx_id != ctx_id) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_last_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            return SPH_ERR_CUDA;
        }
        // the look-up made the device's primary context current if none was
        st = current_context_id(&ctx_id);
        if (st != SPH_OK) return st;
        slot.ptr = static_cast<uint32_t*>(p);
        slot.ctx_id = ctx_id;
    }
    *out = slot.ptr;
    return SPH_OK;
}

}  // namespace
}  // namespace sph

#define NA_TRY(expr)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (expr);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            sph::set_last_error(std::string(#expr) + ": " + cudaGetErrorString(e_));            \
            return SPH_ERR_CUDA;                                                                \
        }                                                                                       \
    } while (0)

extern "C" SPH_API sph_status sph_cell_sort_noalloc(const float* pos, uint32_t n, float h, uint32_t buckets,
                                                    uint32_t* keys, uint32_t* starts, uint32_t* order, void* stream)
{
    using namespace sph;
    if (n > kNoAllocMaxParticles || buckets > kNoAllocMaxBuckets) {
        set_last_error("sph_cell_sort_noalloc: n must be <= 262144 and buckets <= 524288 "
                       "(the fixed scratch array's capacity); use sph_cell_sort for larger inputs");
        return SPH_ERR_CAPACITY;
    }
    if (buckets == 0 || !(h > 0.f) || !starts || (n && (!pos || !keys || !order))) {
        set_last_error("sph_cell_sort_noalloc: null buffer, zero buckets or non-positive h");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if ((reinterpret_cast<uintptr_t>(starts) & 15u) != 0) {   // the scan stores 16 bytes at a time
        set_last_error("sph_cell_sort_noalloc: starts must be 16-byte aligned");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    NA_TRY(cudaStreamIsCapturing(s, &capture));
    if (capture != cudaStreamCaptureStatusNone) {   // the call waits for its status word below
        set_last_error("sph_cell_sort_noalloc: the call is synchronous and cannot be captured into a CUDA graph");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    int device = 0;
    NA_TRY(cudaGetDevice(&device));
    uint32_t* scratch = nullptr;
    sph_status st = scratch_address(device, &scratch);
    if (st != SPH_OK) return st;
    NoAllocArgs a{};
    a.pos = pos;
    a.n = n;
    a.h = h;
    a.fm = make_fastmod(buckets);
    a.buckets = buckets;
    a.keys = keys;
    a.starts = starts;
    a.order = order;
    a.scratch = scratch;
    const uint32_t scan_tiles = (buckets + 1u + kScanTile - 1) / kScanTile;
    const uint32_t clear_blocks = (buckets + 1u + kTileThreads - 1) / kTileThreads;
    k_na_clear<<<clear_blocks, kTileThreads, 0, s>>>(a, scan_tiles);
    NA_TRY(cudaGetLastError());
    const uint32_t blocks = (n + kTileThreads - 1) / kTileThreads;
    if (blocks) {
        k_na_hash_count<<<blocks, kTileThreads, 0, s>>>(a);
        NA_TRY(cudaGetLastError());
    }
    k_na_scan<<<scan_tiles, kScanThreads, 0, s>>>(a);
    NA_TRY(cudaGetLastError());
    if (blocks) {
        k_na_scatter<<<blocks, kTileThreads, 0, s>>>(a);
        NA_TRY(cudaGetLastError());
        k_na_order<<<blocks, kTileThreads, 0, s>>>(a);
        NA_TRY(cudaGetLastError());
    }
    uint32_t err = 0;
    NA_TRY(cudaMemcpyAsync(&err, scratch + kErrOff, sizeof(err), cudaMemcpyDeviceToHost, s));
    NA_TRY(cudaStreamSynchronize(s));
    if (err) {
        set_last_error("sph_cell_sort_noalloc: device status " + std::to_string(err));
        return (err & (DEV_ERR_SCAN_TIMEOUT | DEV_ERR_BARRIER_TIMEOUT)) ? SPH_ERR_DEVICE_TIMEOUT : SPH_ERR_CUDA;
    }
    return SPH_OK;
}
