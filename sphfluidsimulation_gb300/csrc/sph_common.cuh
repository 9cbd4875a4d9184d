// sph_common.cuh -- types and arithmetic shared by the kernels and the host.
//
// Everything here is __host__ __device__ so the host side (table building,
// self-checks) and the kernels use one definition.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <algorithm>

#define SPH_HD __host__ __device__ __forceinline__

namespace sph {

// ---------------------------------------------------------------------------
// Division-free n % d for a divisor fixed per scene.
//
// Granlund & Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), unsigned case with an N+1-bit multiplier:
//   l = ceil(log2 d),  m = floor(2^32 (2^l - d) / d) + 1,
//   t = umulhi(m, n),  q = (t + ((n - t) >> min(l,1))) >> max(l-1, 0).
// Exact for every 32-bit n and 1 <= d < 2^32.  A power-of-two d uses a mask.
// ---------------------------------------------------------------------------
struct FastMod {
    uint32_t d;
    uint32_t m;
    uint32_t sh1;
    uint32_t sh2;
    uint32_t mask;   // d - 1 when d is a power of two, else 0
    uint32_t pow2;   // 1 when d is a power of two
};

inline FastMod make_fastmod(uint32_t d)
{
    FastMod f{};
    f.d = d ? d : 1;
    uint32_t l = 0;
    while (l < 32 && (uint64_t(1) << l) < f.d) ++l;
    f.pow2 = (f.d & (f.d - 1)) == 0;
    f.mask = f.pow2 ? f.d - 1 : 0;
    uint64_t twol = uint64_t(1) << l;
    f.m = uint32_t(((uint64_t(1) << 32) * (twol - f.d)) / f.d + 1);
    f.sh1 = l < 1 ? l : 1;
    f.sh2 = l > 0 ? l - 1 : 0;
    return f;
}

SPH_HD uint32_t umulhi32(uint32_t a, uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return uint32_t((uint64_t(a) * uint64_t(b)) >> 32);
#endif
}

SPH_HD uint32_t fast_mod(uint32_t n, const FastMod& f)
{
    if (f.pow2) return n & f.mask;
    uint32_t t = umulhi32(f.m, n);
    uint32_t q = (t + ((n - t) >> f.sh1)) >> f.sh2;
    return n - q * f.d;
}

// ---------------------------------------------------------------------------
// Cell key (reference SPHFunctions.cpp:65-114).
// ---------------------------------------------------------------------------

// ExpandBits (SF:78-86): spreads the low 10 bits of v to every third bit.
SPH_HD uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Floor (SF:65-76): the C++ engine casts floorf(position / h) to uint32.
// x86-64 g++ converts through int64 and keeps the low 32 bits, so cells wrap
// modulo 2^32 for every |value| < 2^63 (negative ones included); NaN, the
// infinities and larger values give int64's "indefinite" 0x8000000000000000,
// whose low bits are 0.  Written out here, so every host and the device give
// those bits.  x / h is an IEEE division: never built with fast math.
SPH_HD uint32_t cell_coord(float x, float h)
{
    const float f = floorf(x / h);
    return (f >= -9223372036854775808.f && f < 9223372036854775808.f) ? (uint32_t)(int64_t)f : 0u;
}

// Morton3D (SF:88-97) of a cell: x in bit 0, y in bit 1, z in bit 2.
SPH_HD uint32_t morton_cell(uint32_t cx, uint32_t cy, uint32_t cz)
{
    return expand_bits(cx & 0x3FFu) + expand_bits(cy & 0x3FFu) * 2u + expand_bits(cz & 0x3FFu) * 4u;
}

SPH_HD uint32_t cell_hash(float x, float y, float z, float h)
{
    return morton_cell(cell_coord(x, h), cell_coord(y, h), cell_coord(z, h));
}

// ---------------------------------------------------------------------------
// Per-scene descriptor.  Global index spaces:
//   particle slots   [p_off, p_off + n)           (sorted dynamic particles)
//   dynamic buckets  [q_off, q_off + buckets]     (buckets = 2n, +1 sentinel)
//   static slots     [s_off, s_off + s)
//   static buckets   [sq_off, sq_off + s]         (s buckets, +1 sentinel)
// Bucket tables hold a global exclusive scan, so the slot range of local
// bucket b is [start[q_off+b], start[q_off+b+1]) shifted by
// p_off - start[q_off].
// ---------------------------------------------------------------------------
struct SceneDesc {
    uint32_t p_off, n;
    uint32_t q_off, buckets;
    uint32_t s_off, s;
    uint32_t sq_off, t;
    uint32_t t_off;
    uint32_t reorder;              // 1: this step's sort renumbers buffer tags (SimulationEngineCPU.cpp:290-303)
    uint32_t sf_off, sf_buckets;   // neighbour-pass static table (power of two >= 8 s)
    uint32_t sbm_off, sbm_mask;    // static-presence bitmap: word offset, bit-index mask
    FastMod fm_b;
    FastMod fm_s;
    FastMod fm_sf;
    float h, h2;
    float mass, gas;
    float rho0, visc;
    float gx, gy, gz;
    float self_density;
    float kc;       // smoothing kernel constant 15 / (3.1415 h^6)
    float dt;
    // triangle cells (t > 0 and tg_nx > 0): cell (x, y, z) of point p is
    // floor((p - tg_o) * tg_inv); its triangles are tri_list[tri_cells[c] ..
    // tri_cells[c + 1]) with c = tg_cell_off + (z * tg_ny + y) * tg_nx + x
    float tg_ox, tg_oy, tg_oz, tg_inv;
    uint32_t tg_nx, tg_ny, tg_nz, tg_cell_off;
};

// Reach of a boundary triangle: CalculateTriangleForce returns zero beyond
// this distance (SF:209, 219-220).
constexpr float kTriangleReach = 2.5f;

// A tile: up to one CTA's worth of consecutive slots of one scene.
struct Tile {
    uint32_t scene;
    uint32_t begin;
    uint32_t end;
    uint32_t pad;
};

// Size of the static table the neighbour passes use: a power of two of at
// least 8 s buckets, so aliasing between distant wall cells is rare.  The
// reference's own s-bucket table (SimulationEngineCPU.cpp:468) is kept too,
// for readback.
inline uint32_t fast_static_buckets(uint32_t s)
{
    if (!s) return 0;
    uint64_t want = std::max<uint64_t>(64, 8ull * s);
    uint64_t b = 1;
    while (b < want) b <<= 1;
    return (uint32_t)std::min<uint64_t>(b, 1ull << 30);
}

// Bits of a scene's static-presence bitmap: a power of two of about 64 bits
// per static particle (at least 2^12, at most 2^27).  Bit (code & mask) is set
// for every cell within one cell of a static particle, so a particle whose
// own cell's bit is clear has no static neighbour within h.
inline uint32_t static_bitmap_bits(uint32_t s)
{
    if (!s) return 0;
    const uint64_t want = std::min<uint64_t>(std::max<uint64_t>(4096, 64ull * s), 1ull << 27);
    uint64_t b = 1;
    while (b < want) b <<= 1;
    return (uint32_t)b;
}

// Smoothing kernel constant and self density (SF:115-125 as used by
// SimulationEngineCPU.cpp:406-407), evaluated in float with the reference's
// operation order.
inline float kernel_constant(float h)
{
    volatile float d = 3.1415f;
    d = d * h; d = d * h; d = d * h; d = d * h; d = d * h; d = d * h;
    return 15.0f / d;
}

inline float self_density(float mass, float h, float kc)
{
    volatile float w = h * h;
    w = w * h;
    volatile float r = mass * w;
    r = r * kc;
    return r;
}

// Device status word bits.
enum : uint32_t {
    DEV_ERR_SCAN_TIMEOUT = 1u << 0,
    DEV_ERR_BARRIER_TIMEOUT = 1u << 1,
    DEV_ERR_SLOT_RANGE = 1u << 2,
    DEV_ERR_BUCKET_RANGE = 1u << 3,
};

}  // namespace sph
