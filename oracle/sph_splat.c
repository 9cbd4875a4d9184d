/*
 * sph_splat.c -- CPU restatement of the headless particle splat.
 *
 * TEST INFRASTRUCTURE.  Only tests/ load it, to check the CUDA renderer
 * (sph_engine_render) byte for byte.
 *
 * What it restates: the reference's particle renderer
 * (SPHFluidSimulation/source/SPH/Graphics/ParticleRenderer.cpp:75-82), i.e.
 * the vertex shader Shaders/particle.vert:67-117 and the fragment shader
 * Shaders/particle.frag:17-22, evaluated per pixel without a rasteriser:
 *
 *   c      = (V M) (p, 1)                       view-space centre
 *   dist   = |c|, toCamera = -c / dist
 *   right  = cross(toCamera, (0,1,0)) * size    = (-t.z, 0, t.x) * size
 *   up     = (0, size, 0)
 *   color  = mix(u_color, (1,0,0,1), clamp(1 - exp(-pressure / 2000), 0, 1))
 *   color.a *= 1 - smoothstep(5, 4, dist)       (discarded when 0)
 *   r2     = |c - (c + right)|^2
 *
 * A pixel centre is covered when the point q of the quad's plane (through c,
 * spanned by up and right) that projects onto it satisfies |c - q|^2 <= r2,
 * with clip w > 0 and -1 <= z_ndc < 1; q is what perspective-correct
 * interpolation of the quad's vertex positions gives.  Per pixel the smallest
 * (window depth, draw index) wins: depth test LESS, first drawn wins ties.
 * Draw order: dynamic particles in the order given (the reference's buffer
 * order), then static particles.  Particles with a quad corner at clip w <= 0
 * are not drawn.  Every operation is rounded on its own (compiled with
 * -ffp-contract=off), and e^x is computed by the same Cody-Waite reduction
 * and degree-7 Taylor polynomial as the CUDA renderer.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

static float bits_to_float(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t float_to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* e^x: x = k ln2 + r with ln2 = 0.693145751953125 + 1.42860682030941723e-6,
 * e^r by its Taylor polynomial to degree 7, then times 2^k. */
static float exp_splat(float x)
{
    if (!(x > -87.0f)) return x != x ? x : 0.0f;
    if (x > 88.0f) return INFINITY;
    const float k = rintf(x * 1.44269504088896341f);
    float t = k * 0.693145751953125f;
    float r = x - t;
    t = k * 1.42860682030941723e-6f;
    r = r - t;
    float e = 1.0f / 5040.0f;
    e = e * r + 1.0f / 720.0f;
    e = e * r + 1.0f / 120.0f;
    e = e * r + 1.0f / 24.0f;
    e = e * r + 1.0f / 6.0f;
    e = e * r + 0.5f;
    e = e * r + 1.0f;
    e = e * r + 1.0f;
    return e * bits_to_float((uint32_t)(127 + (int)k) << 23);
}

static float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

static float row_dot(const float* m, int r, float x, float y, float z)
{
    float s = m[4 * r] * x;
    s = s + m[4 * r + 1] * y;
    s = s + m[4 * r + 2] * z;
    return s + m[4 * r + 3];
}

typedef struct {
    float cx, cy, cz, rx, rz, up, radius2, dist;
    float color[4];
} splat;

static splat make_splat(const float* mv, float size, const float* u, float x, float y, float z, float pressure)
{
    splat s;
    s.cx = row_dot(mv, 0, x, y, z);
    s.cy = row_dot(mv, 1, x, y, z);
    s.cz = row_dot(mv, 2, x, y, z);
    float d2 = s.cx * s.cx;
    d2 = d2 + s.cy * s.cy;
    d2 = d2 + s.cz * s.cz;
    s.dist = sqrtf(d2);
    const float tx = -s.cx / s.dist, tz = -s.cz / s.dist;
    s.rx = -tz * size;
    s.rz = tx * size;
    s.up = size;
    const float ex = s.cx - (s.cx + s.rx), ey = s.cy - s.cy, ez = s.cz - (s.cz + s.rz);
    float r2 = ex * ex;
    r2 = r2 + ey * ey;
    s.radius2 = r2 + ez * ez;
    const float coef = clamp01(1.0f - exp_splat(-pressure / 2000.0f));
    const float keep = 1.0f - coef;
    s.color[0] = u[0] * keep + coef;
    s.color[1] = u[1] * keep + 0.0f;
    s.color[2] = u[2] * keep + 0.0f;
    s.color[3] = u[3] * keep + coef;
    const float t = clamp01((s.dist - 5.0f) / -1.0f);
    const float sm = (t * t) * (3.0f - 2.0f * t);
    s.color[3] = s.color[3] * (1.0f - sm);
    return s;
}

/* Cramer's rule on [a; b; n] X = (ra, rb, rn), n = (right.z, 0, -right.x). */
static int pixel_point(const float* p, const splat* s, float nx, float ny, float* qx, float* qy, float* qz)
{
    const float a0 = p[0] - nx * p[12], a1 = p[1] - nx * p[13], a2 = p[2] - nx * p[14];
    const float b0 = p[4] - ny * p[12], b1 = p[5] - ny * p[13], b2 = p[6] - ny * p[14];
    const float ra = nx * p[15] - p[3], rb = ny * p[15] - p[7];
    const float n0 = s->rz, n2 = -s->rx;
    const float rn = n0 * s->cx + n2 * s->cz;
    const float det = (a0 * (b1 * n2 - 0.0f) - a1 * (b0 * n2 - b2 * n0)) + a2 * (0.0f - b1 * n0);
    if (det == 0.0f) return 0;
    const float dx = (ra * (b1 * n2) - a1 * (rb * n2 - b2 * rn)) + a2 * (0.0f - b1 * rn);
    const float dy = (a0 * (rb * n2 - b2 * rn) - ra * (b0 * n2 - b2 * n0)) + a2 * (b0 * rn - rb * n0);
    const float dz = (a0 * (b1 * rn) - a1 * (b0 * rn - rb * n0)) + ra * (0.0f - b1 * n0);
    *qx = dx / det;
    *qy = dy / det;
    *qz = dz / det;
    return 1;
}

static void splat_particle(const float* mv, const float* p, uint32_t W, uint32_t H, float size, const float* color,
                           uint64_t* zkey, uint32_t draw, float x, float y, float z, float pressure)
{
    const splat s = make_splat(mv, size, color, x, y, z, pressure);
    if (s.color[3] == 0.0f || !(s.dist > 0.0f)) return;
    float xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
    const float Wf = (float)W, Hf = (float)H;
    for (int k = 0; k < 4; ++k) {
        const float su = (k & 2) ? -1.0f : 1.0f, sr = (k & 1) ? 1.0f : -1.0f;
        const float vx = s.cx + sr * s.rx, vy = s.cy + su * s.up, vz = s.cz + sr * s.rz;
        const float cw = row_dot(p, 3, vx, vy, vz);
        if (!(cw > 0.0f)) return;
        const float wx = ((row_dot(p, 0, vx, vy, vz) / cw) * 0.5f + 0.5f) * Wf;
        const float wy = ((row_dot(p, 1, vx, vy, vz) / cw) * 0.5f + 0.5f) * Hf;
        xmin = fminf(xmin, wx); xmax = fmaxf(xmax, wx);
        ymin = fminf(ymin, wy); ymax = fmaxf(ymax, wy);
    }
    const float fx0 = fmaxf(ceilf(xmin - 0.5f), 0.0f), fx1 = fminf(floorf(xmax - 0.5f), Wf - 1.0f);
    const float fy0 = fmaxf(ceilf(ymin - 0.5f), 0.0f), fy1 = fminf(floorf(ymax - 0.5f), Hf - 1.0f);
    if (!(fx0 <= fx1 && fy0 <= fy1)) return;
    for (int py = (int)fy0; py <= (int)fy1; ++py) {
        const float ny = (((float)py + 0.5f) * 2.0f) / Hf - 1.0f;
        for (int px = (int)fx0; px <= (int)fx1; ++px) {
            const float nx = (((float)px + 0.5f) * 2.0f) / Wf - 1.0f;
            float qx, qy, qz;
            if (!pixel_point(p, &s, nx, ny, &qx, &qy, &qz)) continue;
            const float ex = s.cx - qx, ey = s.cy - qy, ez = s.cz - qz;
            float d2 = ex * ex;
            d2 = d2 + ey * ey;
            d2 = d2 + ez * ez;
            if (d2 > s.radius2) continue;
            const float cz = row_dot(p, 2, qx, qy, qz), cw = row_dot(p, 3, qx, qy, qz);
            if (!(cw > 0.0f)) continue;
            const float zn = cz / cw;
            if (!(zn >= -1.0f && zn < 1.0f)) continue;
            const float depth = zn * 0.5f + 0.5f;
            const uint64_t key = ((uint64_t)float_to_bits(depth) << 32) | draw;
            uint64_t* slot = zkey + (size_t)py * W + px;
            if (key < *slot) *slot = key;
        }
    }
}

static uint8_t to_unorm8(float v) { return (uint8_t)floorf(clamp01(v) * 255.0f + 0.5f); }

/* proj, view, model: column-major 4x4.  dyn: n x 4 (x, y, z, pressure) and
 * stat: s x 3, each in draw order; a layer with a NULL colour is not drawn.
 * zkey: scratch of width*height entries.  Outputs as sph_engine_render. */
EXPORT int sph_oracle_splat(const float* proj, const float* view, const float* model, uint32_t W, uint32_t H,
                            const float* dyn, uint32_t n, float dyn_size, const float* dyn_color,
                            const float* stat, uint32_t s, float stat_size, const float* stat_color,
                            uint64_t* zkey, uint8_t* rgba, float* depth)
{
    float mv[16], p[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            float acc = view[0 * 4 + r] * model[c * 4 + 0];
            for (int k = 1; k < 4; ++k) acc = acc + view[k * 4 + r] * model[c * 4 + k];
            mv[4 * r + c] = acc;
            p[4 * r + c] = proj[c * 4 + r];
        }
    const size_t pixels = (size_t)W * H;
    for (size_t i = 0; i < pixels; ++i) zkey[i] = ~(uint64_t)0;
    if (dyn_color)
        for (uint32_t i = 0; i < n; ++i)
            splat_particle(mv, p, W, H, dyn_size, dyn_color, zkey, i, dyn[4 * (size_t)i], dyn[4 * (size_t)i + 1],
                           dyn[4 * (size_t)i + 2], dyn[4 * (size_t)i + 3]);
    if (stat_color)
        for (uint32_t i = 0; i < s; ++i)
            splat_particle(mv, p, W, H, stat_size, stat_color, zkey, (1u << 31) | i, stat[3 * (size_t)i],
                           stat[3 * (size_t)i + 1], stat[3 * (size_t)i + 2], 0.0f);
    for (size_t i = 0; i < pixels; ++i) {
        const uint64_t key = zkey[i];
        if (key == ~(uint64_t)0) {
            if (rgba) memset(rgba + 4 * i, 0, 4);
            if (depth) depth[i] = 1.0f;
            continue;
        }
        const uint32_t draw = (uint32_t)key, idx = draw & 0x7fffffffu;
        splat q;
        if (draw >> 31)
            q = make_splat(mv, stat_size, stat_color, stat[3 * (size_t)idx], stat[3 * (size_t)idx + 1],
                           stat[3 * (size_t)idx + 2], 0.0f);
        else
            q = make_splat(mv, dyn_size, dyn_color, dyn[4 * (size_t)idx], dyn[4 * (size_t)idx + 1],
                           dyn[4 * (size_t)idx + 2], dyn[4 * (size_t)idx + 3]);
        if (rgba)
            for (int k = 0; k < 4; ++k) rgba[4 * i + k] = to_unorm8(q.color[k]);
        if (depth) depth[i] = bits_to_float((uint32_t)(key >> 32));
    }
    return 0;
}
