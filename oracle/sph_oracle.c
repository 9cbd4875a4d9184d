/*
 * sph_oracle.c -- CPU restatement of the reference SPH step.
 *
 * TEST INFRASTRUCTURE.  This file is the parity oracle and the timed CPU
 * baseline ("port").  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * legs load it; the CUDA engine never links or calls it.
 *
 * What it restates (paths relative to the reference project
 * Murk42/SPHFluidSimulation):
 *   SF   = SPHFluidSimulation/source/SPH/Kernels/SPHFunctions.cpp
 *   ECPU = SPHFluidSimulation/source/SPH/SimulationEngines/SimulationEngineCPU.cpp
 *   SEH  = SPHFluidSimulation/include/SPH/Core/SimulationEngine.h
 *   TPTM = SPHFluidSimulation/source/SPH/Concurrency/ThreadParallelTaskManager.cpp
 *
 * The floating-point expressions keep the reference's operand order and are
 * compiled with -ffp-contract=off, so with REAL=float the results are
 * bit-identical to the reference's own CPU path built the same way (checked
 * against the reference compiled from source, see oracle/ref_harness.cpp).
 * Built with -DSPH_ORACLE_DOUBLE the same code runs in double precision: that
 * is the FP64 rerun used to state the FP32 error of both engines.
 *
 * Threading mirrors the reference engine: thread_count == 0 runs everything
 * synchronously on the caller (deterministic, TPTM EnqueueTask with no pool),
 * thread_count == T > 0 splits particles [N*t/T, N*(t+1)/T) over T threads with
 * barriers between passes and atomic bucket counters (ECPU:132-349).
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#ifdef SPH_ORACLE_DOUBLE
typedef double real;
#define RSQRT(x) sqrt(x)
#define RFLOOR(x) floor(x)
#define RFABS(x) fabs(x)
#else
typedef float real;
/* sqrt of a float computed in double and rounded back equals sqrtf(). */
#define RSQRT(x) sqrtf(x)
#define RFLOOR(x) floorf(x)
#define RFABS(x) fabsf(x)
#endif

#define EXPORT __attribute__((visibility("default")))

/* ---- particle layouts (SF:12-41) ------------------------------------- */

/* DynamicParticle: position, pressure, velocity, hash (SF:12-16). For the
 * float build this is the reference's 32-byte layout byte for byte. */
typedef struct {
    real px, py, pz, pressure;
    real vx, vy, vz;
#ifdef SPH_ORACLE_DOUBLE
    uint32_t hash;
    uint32_t pad_;
#else
    uint32_t hash;
#endif
} dyn_particle;

/* StaticParticle: position and an unused pressure slot (SF:18-21). */
typedef struct {
    real px, py, pz, pressure;
} static_particle;

/* ParticleBehaviourParameters (SF:23-41). */
typedef struct {
    real particleMass, gasConstant, elasticity, viscosity;
    real gravityX, gravityY, gravityZ;
    real restDensity, maxInteractionDistance;
    real selfDensity, smoothingKernelConstant;
} behaviour_params;

typedef struct { real x, y, z; } vec3;

/* ---- hash (SF:65-114) -------------------------------------------------- */

/* Floor(): the C++ engine casts floor(v) from float to uint directly
 * (SF:70-74), which C++ leaves undefined for negative and out-of-range
 * values.  x86-64 g++ compiles the cast as a conversion to int64 followed by
 * truncation to 32 bits: cells wrap modulo 2^32 for every |v| < 2^63, and
 * NaN, the infinities and larger values give the conversion's "indefinite"
 * 0x8000000000000000, whose low 32 bits are 0.  Those steps are written out
 * here, so every host (x86-64 and aarch64 alike) produces the same bits.
 * (The OpenCL side converts to int first, SF:67-68, which agrees for
 * |v| < 2^31.) */
static inline uint32_t floor_to_cell(real v)
{
    const real f = RFLOOR(v);
    return (f >= (real)-9223372036854775808.0 && f < (real)9223372036854775808.0) ? (uint32_t)(int64_t)f : 0u;
}

/* ExpandBits (SF:78-86): spread the low 10 bits of v to every third bit. */
static inline uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

/* Morton3D (SF:88-97): 10 bits per axis, x in bit 0. */
static inline uint32_t morton3d(uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t xx = expand_bits(x & 0x3FFu);
    uint32_t yy = expand_bits(y & 0x3FFu);
    uint32_t zz = expand_bits(z & 0x3FFu);
    return xx + yy * 2u + zz * 4u;
}

typedef struct { uint32_t x, y, z; } cell3;

/* GetCell (SF:99-102): Floor(position / h), a true per-component divide. */
static inline cell3 get_cell(real x, real y, real z, real h)
{
    cell3 c = { floor_to_cell(x / h), floor_to_cell(y / h), floor_to_cell(z / h) };
    return c;
}

/* GetHash (SF:103-114). */
static inline uint32_t get_hash(cell3 c) { return morton3d(c.x, c.y, c.z); }

/* ---- smoothing kernels (SF:115-139) ----------------------------------- */

static inline real kernel_constant(real h)
{
    return (real)15.0 / ((real)3.1415f * h * h * h * h * h * h);
}
static inline real kernel_d0(real r, real h)
{
    if (r >= h) return 0;
    return (h - r) * (h - r) * (h - r);
}
static inline real kernel_d1(real r, real h)
{
    if (r >= h) return 0;
    return -3 * (h - r) * (h - r);
}
static inline real kernel_d2(real r, real h)
{
    if (r >= h) return 0;
    return 6 * (h - r);
}

/* Noise / RandomDirection (SF:140-155).  In the C++ build sin/cos/sqrt of a
 * float resolve to the double functions, and modf(double, float*) returns the
 * fractional part.  RandomDirection stores sin, cos and the square root in
 * float variables (SF:151-153) and multiplies them in float (SF:154); the
 * arithmetic below follows those conversions.  (The FP64 rerun keeps real.) */
static inline float noise(float x)
{
    double ip;
    return (float)modf(sin((double)(x * 112.9898f)) * (double)43758.5453f, &ip);
}
static inline vec3 random_direction(float x)
{
    float theta = noise(x) * 2 * 3.1415f;
    float z = noise(x) * 2 - 1;
    real s = (real)sin((double)theta);
    real c = (real)cos((double)theta);
    real z2 = (real)sqrt((double)(1 - z * z));
    vec3 d = { z2 * c, z2 * s, (real)z };
    return d;
}

/* ---- triangle boundary force (SF:156-223) ----------------------------- */

static inline real dot3(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec3 sub3(vec3 a, vec3 b) { vec3 r = { a.x - b.x, a.y - b.y, a.z - b.z }; return r; }
static inline vec3 add3(vec3 a, vec3 b) { vec3 r = { a.x + b.x, a.y + b.y, a.z + b.z }; return r; }
static inline vec3 mul3(vec3 a, real s) { vec3 r = { a.x * s, a.y * s, a.z * s }; return r; }
static inline vec3 div3(vec3 a, real s) { vec3 r = { a.x / s, a.y / s, a.z / s }; return r; }

/* ClosestPointOnTriangle (SF:156-201), Ericson's region test. */
static vec3 closest_point_on_triangle(vec3 p, vec3 a, vec3 b, vec3 c)
{
    vec3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
    real d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0 && d2 <= 0) return a;
    vec3 bp = sub3(p, b);
    real d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0 && d4 <= d3) return b;
    vec3 cp = sub3(p, c);
    real d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0 && d5 <= d6) return c;
    real vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        real v = d1 / (d1 - d3);
        return add3(a, mul3(ab, v));
    }
    real vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
        real v = d2 / (d2 - d6);
        return add3(a, mul3(ac, v));
    }
    real va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        real v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return add3(b, mul3(sub3(c, b), v));
    }
    real denom = 1 / (va + vb + vc);
    real v = vb * denom;
    real w = vc * denom;
    return add3(add3(a, mul3(ab, v)), mul3(ac, w));
}

/* CalculateTriangleForce (SF:202-223): range 2.5, amplitude (1/x-1)^2 * 50. */
static vec3 triangle_force(vec3 p, const real* tri)
{
    const real range = (real)2.5f;
    vec3 a = { tri[0], tri[1], tri[2] }, b = { tri[3], tri[4], tri[5] }, c = { tri[6], tri[7], tri[8] };
    vec3 to = sub3(closest_point_on_triangle(p, a, b, c), p);
    real dist = RSQRT(dot3(to, to));
    vec3 neg = { -to.x, -to.y, -to.z };
    vec3 dir = div3(neg, dist);
    if (dist > range) { vec3 z = { 0, 0, 0 }; return z; }
    real t = 1 / (dist / range) - 1;
    real amp = t * t;
    return mul3(mul3(dir, amp), (real)50);
}

/* ---- engine state ------------------------------------------------------ */

typedef struct sph_oracle {
    int thread_count;            /* 0 = synchronous (reference threadCount 0) */
    behaviour_params params;

    uint32_t n, s, t;            /* dynamic, static, triangle counts */
    uint32_t buckets;            /* dynamic bucket count B = 2N (ECPU:486) */

    dyn_particle* buffers[3];    /* 3-buffer ring (ECPU:491) */
    uint32_t current;            /* ring index read by the next step */
    _Atomic uint32_t* hash_map;  /* B+1 entries, hash_map[B] = N (ECPU:486-487) */
    uint32_t* particle_map;      /* N entries */
    uint32_t* init_order;        /* slot -> input index after the init sort */
    uint32_t* ident;             /* slot of the current buffer -> input index (bookkeeping only:
                                    the reference keeps no identity; reorders permute it) */
    uint32_t* ident_tmp;

    static_particle* statics;    /* bucket-sorted static particles */
    uint32_t* static_map;        /* S+1 entries (ECPU:468) */
    real* triangles;             /* 9 reals per triangle */

    real reorder_interval;       /* reorderTimeInterval, FLT_MAX = never */
    real reorder_elapsed;
    int parallel_partial_sum;
    _Atomic uint32_t* group_sums;
    double sim_time;

    /* optional debug output: acceleration of the last step, slot order */
    real* accel;

    /* threaded execution */
    pthread_barrier_t barrier;
} sph_oracle;

typedef struct {
    sph_oracle* o;
    uint32_t tid, nthreads;
    real dt;
    uint32_t steps;
    int reorder;
} worker_arg;

static void sync_threads(sph_oracle* o, uint32_t nthreads)
{
    if (nthreads > 1) pthread_barrier_wait(&o->barrier);
}

/* ---- per-particle passes ---------------------------------------------- */

/* UpdateParticlePressure (SF:358-501). */
static void pressure_pass(const sph_oracle* o, uint32_t i, const dyn_particle* in, dyn_particle* out)
{
    const behaviour_params* P = &o->params;
    const real h = P->maxInteractionDistance;
    const dyn_particle* self = in + i;
    real px = self->px, py = self->py, pz = self->pz;
    cell3 c = get_cell(px, py, pz, h);
    real dsum = 0, ssum = 0;
    for (uint32_t ox = c.x - 1u; ox != c.x + 2u; ++ox)
        for (uint32_t oy = c.y - 1u; oy != c.y + 2u; ++oy)
            for (uint32_t oz = c.z - 1u; oz != c.z + 2u; ++oz) {
                cell3 oc = { ox, oy, oz };
                uint32_t hash = get_hash(oc);
                uint32_t b = hash % o->buckets;
                uint32_t begin = atomic_load_explicit(&o->hash_map[b], memory_order_relaxed);
                uint32_t end = atomic_load_explicit(&o->hash_map[b + 1], memory_order_relaxed);
                for (uint32_t k = begin; k < end; ++k) {
                    const dyn_particle* other = in + o->particle_map[k];
                    if (other == self) continue;
                    real dx = other->px - px, dy = other->py - py, dz = other->pz - pz;
                    real d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 > h * h) continue;
                    real d = RSQRT(d2);
                    dsum += kernel_d0(d, h);
                }
                if (o->s == 0) continue;
                b = hash % o->s;
                begin = o->static_map[b];
                end = o->static_map[b + 1];
                for (uint32_t k = begin; k < end; ++k) {
                    const static_particle* other = o->statics + k;
                    real dx = other->px - px, dy = other->py - py, dz = other->pz - pz;
                    real d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 > h * h) continue;
                    real d = RSQRT(d2);
                    ssum += kernel_d0(d, h);
                }
            }
    real density = P->selfDensity + (dsum * P->particleMass + ssum * P->particleMass) * P->smoothingKernelConstant;
    out[i].pressure = P->gasConstant * (density - P->restDensity);
}

/* UpdateParticleDynamics (SF:503-656). */
static void dynamics_pass(const sph_oracle* o, uint32_t i, const dyn_particle* in, dyn_particle* out, real dt)
{
    const behaviour_params* P = &o->params;
    const real h = P->maxInteractionDistance;
    vec3 pos = { in[i].px, in[i].py, in[i].pz };
    real pressure = out[i].pressure;
    vec3 vel = { in[i].vx, in[i].vy, in[i].vz };
    cell3 c = get_cell(pos.x, pos.y, pos.z, h);

    vec3 dynP = { 0, 0, 0 }, dynV = { 0, 0, 0 }, stP = { 0, 0, 0 }, stV = { 0, 0, 0 };
    real density = pressure / P->gasConstant + P->restDensity;

    for (uint32_t ox = c.x - 1u; ox != c.x + 2u; ++ox)
        for (uint32_t oy = c.y - 1u; oy != c.y + 2u; ++oy)
            for (uint32_t oz = c.z - 1u; oz != c.z + 2u; ++oz) {
                cell3 oc = { ox, oy, oz };
                uint32_t hash = get_hash(oc);
                uint32_t b = hash % o->buckets;
                uint32_t begin = atomic_load_explicit(&o->hash_map[b], memory_order_relaxed);
                uint32_t end = atomic_load_explicit(&o->hash_map[b + 1], memory_order_relaxed);
                for (uint32_t k = begin; k < end; ++k) {
                    uint32_t j = o->particle_map[k];
                    if (j == i) continue;
                    real opress = out[j].pressure;
                    vec3 opos = { in[j].px, in[j].py, in[j].pz };
                    vec3 ovel = { in[j].vx, in[j].vy, in[j].vz };
                    vec3 dir = sub3(opos, pos);
                    real d2 = dot3(dir, dir);
                    if (d2 > h * h) continue;
                    real d = RSQRT(d2);
                    if (d2 == 0 || d == 0)
                        dir = random_direction((float)i);
                    else
                        dir = div3(dir, d);
                    dynP = add3(dynP, mul3(mul3(dir, pressure + opress), kernel_d1(d, h)));
                    dynV = add3(dynV, mul3(sub3(ovel, vel), kernel_d2(d, h)));
                }
                if (o->s == 0) continue;
                b = hash % o->s;
                begin = o->static_map[b];
                end = o->static_map[b + 1];
                for (uint32_t k = begin; k < end; ++k) {
                    vec3 opos = { o->statics[k].px, o->statics[k].py, o->statics[k].pz };
                    vec3 dir = sub3(opos, pos);
                    real d2 = dot3(dir, dir);
                    if (d2 > h * h) continue;
                    real d = RSQRT(d2);
                    if (d2 == 0 || d == 0)
                        dir = random_direction((float)i);
                    else
                        dir = div3(dir, d);
                    stP = add3(stP, mul3(mul3(dir, RFABS(pressure)), kernel_d1(d, h)));
                    vec3 nv = { -vel.x, -vel.y, -vel.z };
                    stV = add3(stV, mul3(nv, kernel_d2(d, h)));
                }
            }

    dynP = mul3(dynP, P->particleMass / (2 * density) * P->smoothingKernelConstant);
    dynV = mul3(dynV, P->viscosity * P->particleMass * P->smoothingKernelConstant);
    stP = mul3(stP, P->particleMass / (2 * density) * P->smoothingKernelConstant * (real)1.0f);
    stV = mul3(stV, P->viscosity * P->particleMass * P->smoothingKernelConstant * (real)0.0f);

    vec3 force = { 0, 0, 0 };
    force = add3(force, dynP);
    force = add3(force, dynV);
    force = add3(force, stP);
    force = add3(force, stV);
    for (uint32_t t = 0; t < o->t; ++t)
        force = add3(force, triangle_force(pos, o->triangles + 9 * (size_t)t));
    vec3 g = { P->gravityX, P->gravityY, P->gravityZ };
    vec3 acc = add3(div3(force, density), g);

    if (o->accel) {
        o->accel[3 * (size_t)i + 0] = acc.x;
        o->accel[3 * (size_t)i + 1] = acc.y;
        o->accel[3 * (size_t)i + 2] = acc.z;
    }

    vel = add3(vel, mul3(acc, dt));
    pos = add3(pos, mul3(vel, dt));

    c = get_cell(pos.x, pos.y, pos.z, h);
    uint32_t hash = get_hash(c) % o->buckets;

    out[i].px = pos.x; out[i].py = pos.y; out[i].pz = pos.z;
    out[i].pressure = pressure;
    out[i].vx = vel.x; out[i].vy = vel.y; out[i].vz = vel.z;
    out[i].hash = hash;
}

/* ---- step orchestration: SimulateParticlesTimeStep (ECPU:132-349) ----- */

static void simulate_steps(sph_oracle* o, uint32_t tid, uint32_t nthreads, real dt, uint32_t steps, int reorder)
{
    const uint32_t n = o->n, B = o->buckets;
    const uint32_t begin = (uint32_t)((uint64_t)n * tid / nthreads);
    const uint32_t end = (uint32_t)((uint64_t)n * (tid + 1) / nthreads);
    const uint32_t hbegin = (uint32_t)((uint64_t)B * tid / nthreads);
    const uint32_t hend = (uint32_t)((uint64_t)B * (tid + 1) / nthreads);

    for (uint32_t step = 0; step < steps; ++step) {
        /* ECPU:142-151: read current, advance, write next.  Every thread
         * derives the same ring indices, so no shared state is needed. */
        dyn_particle* in = o->buffers[o->current];
        dyn_particle* out = o->buffers[(o->current + 1) % 3];
        dyn_particle* ordered = o->buffers[(o->current + 2) % 3];
        sync_threads(o, nthreads);

        for (uint32_t i = begin; i < end; ++i) pressure_pass(o, i, in, out);      /* ECPU:162-178 */
        sync_threads(o, nthreads);
        for (uint32_t i = begin; i < end; ++i) dynamics_pass(o, i, in, out, dt);  /* ECPU:182-199 */
        sync_threads(o, nthreads);

        for (uint32_t k = hbegin; k < hend; ++k)                                   /* ECPU:203-204 */
            atomic_store_explicit(&o->hash_map[k], 0u, memory_order_relaxed);
        if (o->group_sums) atomic_store(&o->group_sums[tid], 0u);                 /* ECPU:206-207 */
        sync_threads(o, nthreads);

        for (uint32_t i = begin; i < end; ++i)                                     /* ECPU:211-212 */
            atomic_fetch_add_explicit(&o->hash_map[out[i].hash], 1u, memory_order_relaxed);
        sync_threads(o, nthreads);

        if (!o->group_sums) {                                                      /* ECPU:245-253 */
            if (tid == 0) {
                uint32_t sum = 0;
                for (uint32_t k = 0; k < B; ++k) {
                    sum += atomic_load_explicit(&o->hash_map[k], memory_order_relaxed);
                    atomic_store_explicit(&o->hash_map[k], sum, memory_order_relaxed);
                }
            }
        } else {                                                                   /* ECPU:256-276 */
            uint32_t sum = 0;
            for (uint32_t k = hbegin; k < hend; ++k) {
                sum += atomic_load_explicit(&o->hash_map[k], memory_order_relaxed);
                atomic_store_explicit(&o->hash_map[k], sum, memory_order_relaxed);
            }
            for (uint32_t k = tid; k + 1 < nthreads; ++k)
                atomic_fetch_add(&o->group_sums[k], sum);
            sync_threads(o, nthreads);
            if (tid != 0) {
                uint32_t add = atomic_load(&o->group_sums[tid - 1]);
                for (uint32_t k = hbegin; k < hend; ++k)
                    atomic_fetch_add_explicit(&o->hash_map[k], add, memory_order_relaxed);
            }
        }
        sync_threads(o, nthreads);

        if (reorder) {                                                             /* SF:332-345 */
            for (uint32_t i = begin; i < end; ++i) {
                uint32_t slot = atomic_fetch_sub_explicit(&o->hash_map[out[i].hash], 1u, memory_order_relaxed) - 1u;
                o->particle_map[i] = i;
                ordered[slot] = out[i];
                o->ident_tmp[slot] = o->ident[i];
            }
            sync_threads(o, nthreads);
            if (tid == 0) { uint32_t* t = o->ident; o->ident = o->ident_tmp; o->ident_tmp = t; }
        } else {                                                                   /* SF:346-356 */
            for (uint32_t i = begin; i < end; ++i) {
                uint32_t slot = atomic_fetch_sub_explicit(&o->hash_map[out[i].hash], 1u, memory_order_relaxed) - 1u;
                o->particle_map[slot] = i;
            }
        }
        sync_threads(o, nthreads);
        if (tid == 0) o->current = (o->current + (reorder ? 2u : 1u)) % 3u;
        sync_threads(o, nthreads);
    }
}

static void* worker_main(void* p)
{
    worker_arg* a = (worker_arg*)p;
    simulate_steps(a->o, a->tid, a->nthreads, a->dt, a->steps, a->reorder);
    return NULL;
}

/* ---- public entry points ------------------------------------------------ */

EXPORT sph_oracle* sph_oracle_create(int thread_count)
{
    sph_oracle* o = (sph_oracle*)calloc(1, sizeof(sph_oracle));
    if (!o) return NULL;
    o->thread_count = thread_count < 0 ? 0 : thread_count;
    o->reorder_interval = (real)FLT_MAX;
    return o;
}

static void release(sph_oracle* o)
{
    for (int k = 0; k < 3; ++k) { free(o->buffers[k]); o->buffers[k] = NULL; }
    free(o->hash_map); o->hash_map = NULL;
    free(o->particle_map); o->particle_map = NULL;
    free(o->init_order); o->init_order = NULL;
    free(o->ident); o->ident = NULL;
    free(o->ident_tmp); o->ident_tmp = NULL;
    free(o->statics); o->statics = NULL;
    free(o->static_map); o->static_map = NULL;
    free(o->triangles); o->triangles = NULL;
    free(o->group_sums); o->group_sums = NULL;
    free(o->accel); o->accel = NULL;
    o->n = o->s = o->t = o->buckets = 0;
    o->current = 0;
    o->sim_time = 0;
    o->reorder_elapsed = 0;
    o->reorder_interval = (real)FLT_MAX;
    o->parallel_partial_sum = 0;
}

EXPORT void sph_oracle_destroy(sph_oracle* o)
{
    if (!o) return;
    release(o);
    free(o);
}

/* Static particles: GenerateHashMapAndReorderParticles (SEH:78-114) with
 * S+1 buckets, key = hash % S; the scatter walks particles in index order and
 * decrements, so a bucket lists its members in descending input order. */
static void init_static(sph_oracle* o, const float* pos, uint32_t S)
{
    const real h = o->params.maxInteractionDistance;
    o->s = S;
    if (S == 0) return;
    o->static_map = (uint32_t*)calloc((size_t)S + 1, sizeof(uint32_t));
    o->statics = (static_particle*)calloc(S, sizeof(static_particle));
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * S);
    for (uint32_t i = 0; i < S; ++i) {
        cell3 c = get_cell((real)pos[3 * (size_t)i], (real)pos[3 * (size_t)i + 1], (real)pos[3 * (size_t)i + 2], h);
        keys[i] = get_hash(c) % S;
        ++o->static_map[keys[i]];
    }
    uint32_t sum = 0;
    for (uint32_t k = 0; k <= S; ++k) { sum += o->static_map[k]; o->static_map[k] = sum; }
    for (uint32_t i = 0; i < S; ++i) {
        uint32_t slot = --o->static_map[keys[i]];
        static_particle sp = { (real)pos[3 * (size_t)i], (real)pos[3 * (size_t)i + 1], (real)pos[3 * (size_t)i + 2], 0 };
        o->statics[slot] = sp;
    }
    free(keys);
}

/* Dynamic particles: InitializeDynamicParticles (ECPU:478-504) followed by
 * CalculateHashAndParticleMap (ECPU:55-131): hash + count, serial inclusive
 * scan, then ReorderDynamicParticlesAndFinishHashMap into buffer 1. */
static void init_dynamic(sph_oracle* o, const float* pos, const float* vel, uint32_t N)
{
    const real h = o->params.maxInteractionDistance;
    o->n = N;
    if (N == 0) return;
    o->buckets = 2u * N;
    const uint32_t B = o->buckets;
    o->hash_map = (_Atomic uint32_t*)calloc((size_t)B + 1, sizeof(uint32_t));
    atomic_store(&o->hash_map[B], N);
    o->particle_map = (uint32_t*)calloc(N, sizeof(uint32_t));
    o->init_order = (uint32_t*)calloc(N, sizeof(uint32_t));
    o->ident = (uint32_t*)calloc(N, sizeof(uint32_t));
    o->ident_tmp = (uint32_t*)calloc(N, sizeof(uint32_t));
    for (int k = 0; k < 3; ++k) o->buffers[k] = (dyn_particle*)calloc(N, sizeof(dyn_particle));

    dyn_particle* initial = o->buffers[0];
    for (uint32_t i = 0; i < N; ++i) {
        initial[i].px = (real)pos[3 * (size_t)i];
        initial[i].py = (real)pos[3 * (size_t)i + 1];
        initial[i].pz = (real)pos[3 * (size_t)i + 2];
        if (vel) {
            initial[i].vx = (real)vel[3 * (size_t)i];
            initial[i].vy = (real)vel[3 * (size_t)i + 1];
            initial[i].vz = (real)vel[3 * (size_t)i + 2];
        }
    }
    /* ComputeDynamicParticlesHashAndPrepareHashMap (SF:321-331) */
    for (uint32_t i = 0; i < N; ++i) {
        cell3 c = get_cell(initial[i].px, initial[i].py, initial[i].pz, h);
        uint32_t key = get_hash(c) % B;
        initial[i].hash = key;
        atomic_fetch_add(&o->hash_map[key], 1u);
    }
    uint32_t sum = 0;                                   /* ECPU:98-103 */
    for (uint32_t k = 0; k < B; ++k) { sum += o->hash_map[k]; o->hash_map[k] = sum; }
    dyn_particle* final_ = o->buffers[1];               /* ECPU:105-108 */
    for (uint32_t i = 0; i < N; ++i) {                  /* SF:332-345 */
        uint32_t slot = atomic_fetch_sub(&o->hash_map[initial[i].hash], 1u) - 1u;
        o->particle_map[i] = i;
        final_[slot] = initial[i];
        o->init_order[slot] = i;
        o->ident[slot] = i;
    }
    o->current = 1;
}

/* Initialize (ECPU:396-419).  params = particleMass, gasConstant, elasticity,
 * viscosity, gravityX, gravityY, gravityZ, restDensity, maxInteractionDistance
 * (the scene's particleBehaviourParameters); the two derived constants are
 * computed here as ECPU:406-407 does.  vel may be NULL (zero velocities, as
 * the reference's scene generator leaves them). */
EXPORT int sph_oracle_init(sph_oracle* o, const float* params9,
                           const float* dyn_pos, const float* dyn_vel, uint32_t N,
                           const float* static_pos, uint32_t S,
                           const float* tris, uint32_t T,
                           float reorder_interval, int parallel_partial_sum)
{
    if (!o) return -1;
    release(o);
    behaviour_params* P = &o->params;
    P->particleMass = params9[0];
    P->gasConstant = params9[1];
    P->elasticity = params9[2];
    P->viscosity = params9[3];
    P->gravityX = params9[4];
    P->gravityY = params9[5];
    P->gravityZ = params9[6];
    P->restDensity = params9[7];
    P->maxInteractionDistance = params9[8];
    P->smoothingKernelConstant = kernel_constant(P->maxInteractionDistance);
    P->selfDensity = P->particleMass * kernel_d0(0, P->maxInteractionDistance) * P->smoothingKernelConstant;
    o->reorder_interval = (real)reorder_interval;
    o->parallel_partial_sum = parallel_partial_sum;
    if (parallel_partial_sum && o->thread_count > 0)
        o->group_sums = (_Atomic uint32_t*)calloc((size_t)o->thread_count, sizeof(uint32_t));
    init_static(o, static_pos, S);
    init_dynamic(o, dyn_pos, dyn_vel, N);
    o->t = T;
    if (T) {
        o->triangles = (real*)malloc(sizeof(real) * 9 * (size_t)T);
        for (size_t k = 0; k < 9 * (size_t)T; ++k) o->triangles[k] = (real)tris[k];
    }
    return 0;
}

/* Update (ECPU:420-459).  The reorder decision is taken once per call and
 * the elapsed time advances by dt per call, as in the reference. */
EXPORT int sph_oracle_update(sph_oracle* o, float dt, uint32_t steps)
{
    if (!o || o->buffers[0] == NULL) return -1;
    if (o->n == 0) return 0;
    int reorder = o->reorder_elapsed > o->reorder_interval;
    uint32_t T = (uint32_t)o->thread_count;
    if (T <= 1) {
        simulate_steps(o, 0, 1, (real)dt, steps, reorder);
    } else {
        pthread_barrier_init(&o->barrier, NULL, T);
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * T);
        worker_arg* args = (worker_arg*)malloc(sizeof(worker_arg) * T);
        for (uint32_t k = 0; k < T; ++k) {
            worker_arg a = { o, k, T, (real)dt, steps, reorder };
            args[k] = a;
            pthread_create(&th[k], NULL, worker_main, &args[k]);
        }
        for (uint32_t k = 0; k < T; ++k) pthread_join(th[k], NULL);
        pthread_barrier_destroy(&o->barrier);
        free(th);
        free(args);
    }
    o->sim_time += (double)dt * steps;
    o->reorder_elapsed += (real)dt;
    if (o->reorder_elapsed > o->reorder_interval) o->reorder_elapsed = 0;
    return 0;
}

/* Enables the per-particle acceleration output (slot order, 3 reals). */
EXPORT void sph_oracle_record_accel(sph_oracle* o, int on)
{
    if (!o) return;
    free(o->accel);
    o->accel = (on && o->n) ? (real*)calloc(3 * (size_t)o->n, sizeof(real)) : NULL;
}

EXPORT uint32_t sph_oracle_count(const sph_oracle* o, int which)
{
    switch (which) {
    case 0: return o->n;
    case 1: return o->s;
    case 2: return o->buckets;
    case 3: return o->t;
    default: return 0;
    }
}

EXPORT double sph_oracle_sim_time(const sph_oracle* o) { return o->sim_time; }

/* Readback of the current buffer (what LockRead returns), widened to double:
 * out = N x 8 (px, py, pz, pressure, vx, vy, vz, hash). */
EXPORT void sph_oracle_read_dynamic(const sph_oracle* o, double* out)
{
    const dyn_particle* cur = o->buffers[o->current];
    for (uint32_t i = 0; i < o->n; ++i) {
        double* r = out + 8 * (size_t)i;
        r[0] = cur[i].px; r[1] = cur[i].py; r[2] = cur[i].pz; r[3] = cur[i].pressure;
        r[4] = cur[i].vx; r[5] = cur[i].vy; r[6] = cur[i].vz; r[7] = (double)cur[i].hash;
    }
}

/* Raw 32-byte particles of the current buffer (float build only). */
EXPORT int sph_oracle_read_raw(const sph_oracle* o, void* out)
{
#ifdef SPH_ORACLE_DOUBLE
    (void)o; (void)out;
    return -1;
#else
    memcpy(out, o->buffers[o->current], sizeof(dyn_particle) * (size_t)o->n);
    return 0;
#endif
}

EXPORT void sph_oracle_read_maps(const sph_oracle* o, uint32_t* hash_map, uint32_t* particle_map, uint32_t* init_order)
{
    if (hash_map) for (uint32_t k = 0; k <= o->buckets && o->n; ++k) hash_map[k] = atomic_load(&o->hash_map[k]);
    if (particle_map) memcpy(particle_map, o->particle_map, sizeof(uint32_t) * (size_t)o->n);
    if (init_order) memcpy(init_order, o->ident, sizeof(uint32_t) * (size_t)o->n);
}

EXPORT void sph_oracle_read_static(const sph_oracle* o, double* pos4, uint32_t* static_map)
{
    for (uint32_t i = 0; i < o->s; ++i) {
        pos4[4 * (size_t)i + 0] = o->statics[i].px;
        pos4[4 * (size_t)i + 1] = o->statics[i].py;
        pos4[4 * (size_t)i + 2] = o->statics[i].pz;
        pos4[4 * (size_t)i + 3] = o->statics[i].pressure;
    }
    if (static_map && o->s) memcpy(static_map, o->static_map, sizeof(uint32_t) * ((size_t)o->s + 1));
}

EXPORT void sph_oracle_read_accel(const sph_oracle* o, double* acc)
{
    if (!o->accel) return;
    for (size_t k = 0; k < 3 * (size_t)o->n; ++k) acc[k] = o->accel[k];
}

EXPORT void sph_oracle_derived(const sph_oracle* o, double* self_density, double* kernel_c)
{
    *self_density = o->params.selfDensity;
    *kernel_c = o->params.smoothingKernelConstant;
}

/* ---- stage functions for stage-wise parity ----------------------------- */

/* key = GetHash(GetCell(p)) % buckets for each position (SF:321-331). */
EXPORT void sph_oracle_hash(const float* pos, uint32_t n, float h, uint32_t buckets, uint32_t* keys)
{
    for (uint32_t i = 0; i < n; ++i) {
        cell3 c = get_cell((real)pos[3 * (size_t)i], (real)pos[3 * (size_t)i + 1], (real)pos[3 * (size_t)i + 2], (real)h);
        keys[i] = get_hash(c) % buckets;
    }
}

/* One counting sort exactly as a synchronous step does it (ECPU:203-316,
 * non-reorder mode): counts, inclusive scan, then the decrementing fill.
 * starts gets buckets+1 entries (starts[buckets] = n), particle_map n. */
EXPORT void sph_oracle_counting_sort(const uint32_t* keys, uint32_t n, uint32_t buckets,
                                     uint32_t* counts, uint32_t* starts, uint32_t* particle_map)
{
    memset(counts, 0, sizeof(uint32_t) * buckets);
    for (uint32_t i = 0; i < n; ++i) ++counts[keys[i]];
    uint32_t sum = 0;
    for (uint32_t k = 0; k < buckets; ++k) { sum += counts[k]; starts[k] = sum; }
    starts[buckets] = n;
    for (uint32_t i = 0; i < n; ++i) particle_map[--starts[keys[i]]] = i;
}
