// sph_render.cu -- headless particle splats.
//
// The reference draws every particle as a camera-facing quad and keeps the
// disc inside it (SPHFluidSimulation/source/SPH/Graphics/ParticleRenderer.cpp:
// 75-82 with Shaders/particle.vert:67-117 and particle.frag:17-22), through
// OpenGL.  There is no graphics stack here, so the same arithmetic runs as two
// CUDA kernels writing an RGBA8 image and a depth image in device memory:
//
//   splat    one thread per particle: view-space centre c = (V M) p, quad
//            half-vectors up = (0, size, 0) and right = cross(-c/|c|, y) size,
//            colour mix(u_color, red, clamp(1 - exp(-p/2000), 0, 1)) with
//            alpha faded by 1 - smoothstep(5, 4, |c|); for every pixel of the
//            quad's screen box, the point q of the quad's plane that projects
//            to the pixel centre (what perspective-correct interpolation of
//            the vertex positions gives) must lie in the disc |q - c|^2 <=
//            |c - (c + right)|^2 and inside the depth range; a 64-bit atomicMin
//            keeps, per pixel, the smallest (depth, draw index): the depth test
//            LESS with the first drawn fragment winning ties;
//   resolve  one thread per pixel: the winner's colour as 8-bit RGBA and the
//            window depth (1 where nothing was drawn).
//
// Draw order is the reference's: dynamic particles by buffer index, then
// static particles in their sorted order.  Every float operation is rounded
// on its own (no contraction), and exp is the routine below, so the CPU
// restatement in oracle/sph_splat.c produces the same bytes.
#include "sph_state.h"

namespace sph {
namespace {

constexpr unsigned long long kEmpty = ~0ull;

struct RenderArgs {
    float mv[16];        // u_viewMatrix * u_modelMatrix, row-major
    float p[16];         // u_projMatrix, row-major
    uint32_t width, height;
    float size[2];       // per layer: u_size
    float color[2][4];   // per layer: u_color
    int enabled[2];
    const float4* dpos;  // dynamic particles, sorted slots (w = input index)
    const float4* dvel;  // w = pressure
    const uint32_t* dtag;
    uint32_t dn;
    const uint32_t* slot_of_tag;
    const float4* spos;  // static particles in the reference's sorted order
    uint32_t sn;
    unsigned long long* zkey;
    uchar4* rgba;
    float* depth;
};

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }

// e^x by Cody-Waite reduction x = k ln2 + r (ln2 split into a short high part
// and the remainder), a degree-7 Taylor polynomial for e^r on |r| <= ln2/2
// (relative error below 2e-7 there) and an exponent shift for 2^k.
__device__ __forceinline__ float exp_splat(float x)
{
    if (!(x > -87.0f)) return x != x ? x : 0.0f;
    if (x > 88.0f) return __int_as_float(0x7f800000);
    const float k = rintf(mul(x, 1.44269504088896341f));
    const float r = sub(sub(x, mul(k, 0.693145751953125f)), mul(k, 1.42860682030941723e-6f));
    float e = 1.0f / 5040.0f;
    e = add(mul(e, r), 1.0f / 720.0f);
    e = add(mul(e, r), 1.0f / 120.0f);
    e = add(mul(e, r), 1.0f / 24.0f);
    e = add(mul(e, r), 1.0f / 6.0f);
    e = add(mul(e, r), 0.5f);
    e = add(mul(e, r), 1.0f);
    e = add(mul(e, r), 1.0f);
    return mul(e, __int_as_float((127 + (int)k) << 23));   // k in -126 .. 127: 2^k is a normal float
}

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// row r of a row-major 4x4 times (x, y, z, 1), summed left to right
__device__ __forceinline__ float row_dot(const float* m, int r, float x, float y, float z)
{
    return add(add(add(mul(m[4 * r], x), mul(m[4 * r + 1], y)), mul(m[4 * r + 2], z)), m[4 * r + 3]);
}

struct Splat {
    float cx, cy, cz;      // view-space centre
    float rx, rz;          // right (its y is 0)
    float up;              // up = (0, size, 0)
    float radius2;
    float dist;
    float4 color;
};

__device__ __forceinline__ Splat make_splat(const RenderArgs& a, int layer, float x, float y, float z, float pressure)
{
    Splat s;
    s.cx = row_dot(a.mv, 0, x, y, z);
    s.cy = row_dot(a.mv, 1, x, y, z);
    s.cz = row_dot(a.mv, 2, x, y, z);
    s.dist = __fsqrt_rn(add(add(mul(s.cx, s.cx), mul(s.cy, s.cy)), mul(s.cz, s.cz)));
    const float tx = dvd(-s.cx, s.dist), tz = dvd(-s.cz, s.dist);
    const float size = a.size[layer];
    s.rx = mul(-tz, size);           // cross(toCamera, (0,1,0)) = (-t.z, 0, t.x)
    s.rz = mul(tx, size);
    s.up = size;
    const float ex = sub(s.cx, add(s.cx, s.rx)), ey = sub(s.cy, s.cy), ez = sub(s.cz, add(s.cz, s.rz));
    s.radius2 = add(add(mul(ex, ex), mul(ey, ey)), mul(ez, ez));
    const float* u = a.color[layer];
    const float coef = clamp01(sub(1.0f, exp_splat(dvd(-pressure, 2000.0f))));
    const float keep = sub(1.0f, coef);
    s.color.x = add(mul(u[0], keep), coef);      // mix(u_color, (1, 0, 0, 1), coef)
    s.color.y = add(mul(u[1], keep), 0.0f);
    s.color.z = add(mul(u[2], keep), 0.0f);
    s.color.w = add(mul(u[3], keep), coef);
    const float t = clamp01(dvd(sub(s.dist, 5.0f), -1.0f));   // smoothstep(5, 4, dist)
    const float sm = mul(mul(t, t), sub(3.0f, mul(2.0f, t)));
    s.color.w = mul(s.color.w, sub(1.0f, sm));
    return s;
}

// The point of the quad's plane (through c, spanned by up and right) whose
// projection is NDC (nx, ny): the plane and the two projective constraints
// (P0 - nx P3).X = nx P3w - P0w and (P1 - ny P3).X = ny P3w - P1w solved by
// Cramer's rule.  False when the system is singular.
__device__ __forceinline__ bool pixel_point(const RenderArgs& a, const Splat& s, float nx, float ny, float& qx,
                                            float& qy, float& qz)
{
    const float* p = a.p;
    const float a0 = sub(p[0], mul(nx, p[12])), a1 = sub(p[1], mul(nx, p[13])), a2 = sub(p[2], mul(nx, p[14]));
    const float b0 = sub(p[4], mul(ny, p[12])), b1 = sub(p[5], mul(ny, p[13])), b2 = sub(p[6], mul(ny, p[14]));
    const float ra = sub(mul(nx, p[15]), p[3]), rb = sub(mul(ny, p[15]), p[7]);
    // plane normal up x right = (right.z, 0, -right.x) (up is along y)
    const float n0 = s.rz, n2 = -s.rx;
    const float rn = add(mul(n0, s.cx), mul(n2, s.cz));
    // det [a; b; n] with n1 = 0
    const float det = add(sub(mul(a0, sub(mul(b1, n2), 0.0f)), mul(a1, sub(mul(b0, n2), mul(b2, n0)))),
                          mul(a2, sub(0.0f, mul(b1, n0))));
    if (det == 0.0f) return false;
    const float dx = add(sub(mul(ra, mul(b1, n2)), mul(a1, sub(mul(rb, n2), mul(b2, rn)))),
                         mul(a2, sub(0.0f, mul(b1, rn))));
    const float dy = add(sub(mul(a0, sub(mul(rb, n2), mul(b2, rn))), mul(ra, sub(mul(b0, n2), mul(b2, n0)))),
                         mul(a2, sub(mul(b0, rn), mul(rb, n0))));
    const float dz = add(sub(mul(a0, mul(b1, rn)), mul(a1, sub(mul(b0, rn), mul(rb, n0)))),
                         mul(ra, sub(0.0f, mul(b1, n0))));
    qx = dvd(dx, det);
    qy = dvd(dy, det);
    qz = dvd(dz, det);
    return true;
}

__device__ void splat_particle(const RenderArgs& a, int layer, uint32_t draw, float x, float y, float z, float pressure)
{
    const Splat s = make_splat(a, layer, x, y, z, pressure);
    if (s.color.w == 0.0f || !(s.dist > 0.0f)) return;     // discarded (particle.frag:19)
    // screen box of the quad's corners c +- up +- right
    float xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
    const float W = (float)a.width, H = (float)a.height;
    for (int k = 0; k < 4; ++k) {
        const float su = (k & 2) ? -1.0f : 1.0f, sr = (k & 1) ? 1.0f : -1.0f;
        const float vx = add(s.cx, mul(sr, s.rx)), vy = add(s.cy, mul(su, s.up)), vz = add(s.cz, mul(sr, s.rz));
        const float cw = row_dot(a.p, 3, vx, vy, vz);
        if (!(cw > 0.0f)) return;                           // a corner behind the eye: not drawn
        const float wx = mul(add(mul(dvd(row_dot(a.p, 0, vx, vy, vz), cw), 0.5f), 0.5f), W);
        const float wy = mul(add(mul(dvd(row_dot(a.p, 1, vx, vy, vz), cw), 0.5f), 0.5f), H);
        xmin = fminf(xmin, wx); xmax = fmaxf(xmax, wx);
        ymin = fminf(ymin, wy); ymax = fmaxf(ymax, wy);
    }
    const float fx0 = fmaxf(ceilf(sub(xmin, 0.5f)), 0.0f), fx1 = fminf(floorf(sub(xmax, 0.5f)), W - 1.0f);
    const float fy0 = fmaxf(ceilf(sub(ymin, 0.5f)), 0.0f), fy1 = fminf(floorf(sub(ymax, 0.5f)), H - 1.0f);
    if (!(fx0 <= fx1 && fy0 <= fy1)) return;
    const int x0 = (int)fx0, x1 = (int)fx1, y0 = (int)fy0, y1 = (int)fy1;
    for (int py = y0; py <= y1; ++py) {
        const float ny = sub(dvd(mul(add((float)py, 0.5f), 2.0f), H), 1.0f);
        for (int px = x0; px <= x1; ++px) {
            const float nx = sub(dvd(mul(add((float)px, 0.5f), 2.0f), W), 1.0f);
            float qx, qy, qz;
            if (!pixel_point(a, s, nx, ny, qx, qy, qz)) continue;
            const float ex = sub(s.cx, qx), ey = sub(s.cy, qy), ez = sub(s.cz, qz);
            if (add(add(mul(ex, ex), mul(ey, ey)), mul(ez, ez)) > s.radius2) continue;   // particle.frag:19
            const float cz = row_dot(a.p, 2, qx, qy, qz), cw = row_dot(a.p, 3, qx, qy, qz);
            if (!(cw > 0.0f)) continue;
            const float zn = dvd(cz, cw);
            if (!(zn >= -1.0f && zn < 1.0f)) continue;         // depth range; the cleared depth is 1
            const float depth = add(mul(zn, 0.5f), 0.5f);
            const unsigned long long key =
                ((unsigned long long)__float_as_uint(depth) << 32) | ((uint32_t)layer << 31) | draw;
            atomicMin(a.zkey + (size_t)py * a.width + px, key);
        }
    }
}

__global__ void k_render_clear(unsigned long long* zkey, size_t count)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        zkey[i] = kEmpty;
}

__global__ void k_slot_of_tag(const uint32_t* tag, uint32_t n, uint32_t* slot_of_tag)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) slot_of_tag[tag[i]] = i;
}

__global__ void __launch_bounds__(128) k_splat(RenderArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (a.enabled[0] && i < a.dn) {
        const float4 p = a.dpos[i];
        splat_particle(a, 0, a.dtag[i], p.x, p.y, p.z, a.dvel[i].w);
    } else if (a.enabled[1] && i >= a.dn && i - a.dn < a.sn) {
        const float4 p = a.spos[i - a.dn];
        splat_particle(a, 1, i - a.dn, p.x, p.y, p.z, 0.0f);   // static pressure is never written
    }
}

__device__ __forceinline__ unsigned char to_unorm8(float v)
{
    return (unsigned char)floorf(add(mul(clamp01(v), 255.0f), 0.5f));
}

__global__ void k_resolve(RenderArgs a)
{
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)a.width * a.height) return;
    const unsigned long long key = a.zkey[i];
    if (key == kEmpty) {
        a.rgba[i] = make_uchar4(0, 0, 0, 0);
        a.depth[i] = 1.0f;
        return;
    }
    const uint32_t draw = (uint32_t)key;
    const int layer = (int)(draw >> 31);
    const uint32_t idx = draw & 0x7fffffffu;
    float4 p;
    float pressure = 0.0f;
    if (layer == 0) {
        const uint32_t slot = a.slot_of_tag[idx];
        p = a.dpos[slot];
        pressure = a.dvel[slot].w;
    } else {
        p = a.spos[idx];
    }
    const Splat s = make_splat(a, layer, p.x, p.y, p.z, pressure);
    a.rgba[i] = make_uchar4(to_unorm8(s.color.x), to_unorm8(s.color.y), to_unorm8(s.color.z), to_unorm8(s.color.w));
    a.depth[i] = __uint_as_float((uint32_t)(key >> 32));
}

// Row-major product of two column-major 4x4 matrices (a b), sums left to right.
void mat_mul_rowmajor(const float* a_col, const float* b_col, float* out_row)
{
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            float s = a_col[0 * 4 + r] * b_col[c * 4 + 0];
            for (int k = 1; k < 4; ++k) s = s + a_col[k * 4 + r] * b_col[c * 4 + k];
            out_row[4 * r + c] = s;
        }
}

}  // namespace

sph_status StepState::render(const sph_render_view& view, const sph_render_layer* dyn, const sph_render_layer* stat,
                             uint8_t* rgba_out, float* depth_out)
{
    if (scenes.empty()) return SPH_ERR_NOT_INITIALIZED;
    if (view.width == 0 || view.height == 0 || (uint64_t)view.width * view.height > (1ull << 28)) {
        set_last_error("image size out of range (1 .. 2^28 pixels)");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    const SceneDesc& d = scenes[0];
    RenderArgs a{};
    mat_mul_rowmajor(view.view, view.model, a.mv);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) a.p[4 * r + c] = view.proj[c * 4 + r];
    a.width = view.width;
    a.height = view.height;
    const sph_render_layer* layers[2] = {dyn, stat};
    for (int l = 0; l < 2; ++l) {
        a.enabled[l] = layers[l] != nullptr;
        if (!layers[l]) continue;
        a.size[l] = layers[l]->size;
        for (int k = 0; k < 4; ++k) a.color[l][k] = layers[l]->color[k];
    }
    a.dpos = pos + d.p_off;
    a.dvel = vel + d.p_off;
    a.dtag = tag + d.p_off;
    a.dn = d.n;
    a.slot_of_tag = tag_io;   // scratch, free between steps
    a.spos = spos_ref + d.s_off;
    a.sn = d.s;
    const size_t pixels = (size_t)view.width * view.height;
    if (pixels > render_pixels_) {
        for (void* p : {(void*)render_zkey_, (void*)render_rgba_, (void*)render_depth_})
            if (p) cudaFree(p);
        render_zkey_ = nullptr;
        render_rgba_ = nullptr;
        render_depth_ = nullptr;
        render_pixels_ = 0;
        sph_status st;
        if ((st = dev_alloc(&render_zkey_, pixels)) != SPH_OK) return st;
        if ((st = dev_alloc(&render_rgba_, pixels)) != SPH_OK) return st;
        if ((st = dev_alloc(&render_depth_, pixels)) != SPH_OK) return st;
        render_pixels_ = pixels;
    }
    a.zkey = render_zkey_;
    a.rgba = render_rgba_;
    a.depth = render_depth_;
    k_render_clear<<<1024, 256, 0, stream_>>>(a.zkey, pixels);
    if (d.n) k_slot_of_tag<<<(d.n + 255) / 256, 256, 0, stream_>>>(a.dtag, d.n, tag_io);
    const uint64_t total = (uint64_t)d.n + d.s;
    if (total) k_splat<<<(unsigned)((total + 127) / 128), 128, 0, stream_>>>(a);
    k_resolve<<<(unsigned)((pixels + 255) / 256), 256, 0, stream_>>>(a);
    CUDA_TRY(cudaGetLastError());
    if (rgba_out)
        CUDA_TRY(cudaMemcpyAsync(rgba_out, render_rgba_, 4 * pixels, cudaMemcpyDeviceToHost, stream_));
    if (depth_out)
        CUDA_TRY(cudaMemcpyAsync(depth_out, render_depth_, sizeof(float) * pixels, cudaMemcpyDeviceToHost, stream_));
    return check_device_error();
}

}  // namespace sph
