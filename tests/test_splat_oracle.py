"""The CPU restatement of the headless particle splat (oracle/sph_splat.c),
checked against the shader arithmetic it restates (particle.vert:67-117,
particle.frag:17-22) on hand-computable cases -- the disc's size on screen,
the pressure colour, the distance fade and the depth test -- and against an
independent float64 restatement of the GL pipeline those shaders run in
(rasterised triangle strip, perspective-correct interpolation), over random
particles and cameras."""
import math

import numpy as np

from oracle_lib import oracle_splat
from sphfluidsimulation_gb300 import render

W = H = 64
PROJ = render.perspective(math.radians(90.0), 1.0, 0.1, 100.0)
EYE = render.identity()


def splat(dyn4, layer=(0.5, (0.2, 0.4, 0.6, 1.0)), stat3=None, stat_layer=None, proj=PROJ):
    stat3 = np.zeros((0, 3), np.float32) if stat3 is None else stat3
    return oracle_splat(proj, EYE, EYE, W, H, np.asarray(dyn4, np.float32), layer, stat3, stat_layer)


def test_disc_size_and_colour():
    # a particle 6 units ahead (beyond the 4-5 unit fade), radius 0.5:
    # f = 1 / tan(45 deg) = 1, so the disc spans 0.5 / 6 * 32 px = 2.67 px
    rgba, depth = splat([[0.0, 0.0, -6.0, 0.0]], layer=(0.5, (0.2, 0.4, 0.6, 1.0)))
    covered = rgba[..., 3] > 0
    r = 0.5 / 6.0 * (W / 2)
    assert abs(covered.sum() - math.pi * r * r) < 2 * math.pi * r + 4
    ys, xs = np.nonzero(covered)
    assert abs(xs.mean() + 0.5 - W / 2) < 0.6 and abs(ys.mean() + 0.5 - H / 2) < 0.6
    assert (rgba[covered] == np.array([51, 102, 153, 255], np.uint8)).all()
    # window depth of the centre: z_ndc = (far + near)/(near - far) + 2 far near / ((near - far) z) ... at z = -6
    n_, f_ = 0.1, 100.0
    zn = ((f_ + n_) / (n_ - f_) * -6.0 + 2 * f_ * n_ / (n_ - f_)) / 6.0
    assert abs(depth[H // 2, W // 2] - (zn * 0.5 + 0.5)) < 1e-5
    assert (depth[~covered] == 1.0).all()


def test_pressure_colour_and_fade():
    # pressure 2000 ln 2: 1 - exp(-p/2000) = 1/2, so the colour is halfway to red
    p = 2000.0 * math.log(2.0)
    rgba, _ = splat([[0.0, 0.0, -6.0, p]], layer=(0.5, (0.0, 0.0, 1.0, 1.0)))
    c = rgba[H // 2, W // 2].astype(int)
    assert np.abs(c - np.array([128, 0, 128, 255])).max() <= 1
    # closer than 4 units the alpha is 0: discarded; at 4.5 it is halfway
    rgba, _ = splat([[0.0, 0.0, -3.0, 0.0]])
    assert rgba[..., 3].max() == 0
    rgba, _ = splat([[0.0, 0.0, -4.5, 0.0]], layer=(0.3, (1.0, 1.0, 1.0, 1.0)))
    assert abs(int(rgba[H // 2, W // 2, 3]) - 128) <= 1


def test_depth_test_and_draw_order():
    # the nearer particle wins wherever they overlap, whatever the order
    near, far = [0.0, 0.0, -6.0, 0.0], [0.1, 0.0, -8.0, 1e6]
    for order in ([near, far], [far, near]):
        rgba, depth = splat(order, layer=(0.5, (0.0, 1.0, 0.0, 1.0)))
        assert tuple(rgba[H // 2, W // 2]) == (0, 255, 0, 255)
    # equal depth: the first drawn stays (depth test LESS)
    a, b = [0.0, 0.0, -6.0, 0.0], [0.0, 0.0, -6.0, 1e6]
    rgba, _ = splat([a, b], layer=(0.5, (0.0, 1.0, 0.0, 1.0)))
    assert tuple(rgba[H // 2, W // 2]) == (0, 255, 0, 255)
    rgba, _ = splat([b, a], layer=(0.5, (0.0, 1.0, 0.0, 1.0)))
    assert tuple(rgba[H // 2, W // 2]) == (255, 0, 0, 255)


def test_static_layer_and_behind_the_eye():
    stat = np.array([[0.0, 0.0, -7.0]], np.float32)
    rgba, _ = splat(np.zeros((0, 4)), stat3=stat, stat_layer=(0.3, (0.0, 0.0, 1.0, 1.0)))
    assert tuple(rgba[H // 2, W // 2]) == (0, 0, 255, 255)
    rgba, _ = splat([[0.0, 0.0, 6.0, 0.0]])    # behind the camera: not drawn
    assert rgba[..., 3].max() == 0


# ---------------------------------------------------------------------------
# An independent restatement in float64: the GL pipeline itself
# ---------------------------------------------------------------------------
#
# The C oracle solves, per pixel, for the point of the quad's plane that
# projects onto the pixel centre (Cramer's rule, float32).  This restatement
# follows the GL pipeline the shaders run in instead, in float64:
#   * particle.vert:67-117: the four corners c +- up +- right, clip
#     positions P (c_k, 1), the pressure colour and the distance fade;
#   * the triangle strip of ParticleRenderer.cpp:75-82 (corners 0 1 2 and
#     2 1 3), rasterised at pixel centres with screen-space barycentrics;
#   * perspective-correct interpolation of f_pos (attribute / w over 1 / w)
#     and window depth interpolated linearly in screen space;
#   * particle.frag:17-22: discard when |f_center - f_pos|^2 > f_radiusSqr
#     or alpha == 0; depth test LESS, the first drawn fragment winning ties.
# Pixels whose result rounding can decide are left out of the comparison:
# a fragment within a relative 1e-4 of its disc's edge, or two covering
# fragments whose depths lie within 1e-6 of each other.

EDGE_REL = 1e-4
DEPTH_TIE = 1e-6
DEPTH_TOL = 5e-7     # window depth, absolute (float32 rounding: measured <= 7.1e-8)
COLOUR_TOL = 1       # RGBA8 steps


def _mat(m16):
    """Column-major float32[16] -> 4x4 float64 acting on column vectors."""
    return np.asarray(m16, np.float64).reshape(4, 4).T


def splat_f64(proj, view, model, width, height, dyn4, dyn_layer, stat3, stat_layer):
    """Returns per pixel (covered, rgba float64 in [0, 1], depth, ambiguous)."""
    P, MV = _mat(proj), _mat(view) @ _mat(model)
    frags = [[] for _ in range(width * height)]     # (depth, draw, rgba, margin)
    draws = []
    if dyn_layer is not None:
        draws += [(np.asarray(d[:3], np.float64), float(d[3]), dyn_layer) for d in np.asarray(dyn4).reshape(-1, 4)]
    if stat_layer is not None:
        draws += [(np.asarray(s, np.float64), 0.0, stat_layer) for s in np.asarray(stat3).reshape(-1, 3)]
    for draw, (p, pressure, (size, ucol)) in enumerate(draws):
        c = (MV @ np.append(p, 1.0))[:3]
        dist = np.linalg.norm(c)
        t = -c / dist
        right = np.cross(t, [0.0, 1.0, 0.0]) * size
        up = np.array([0.0, size, 0.0])
        coef = min(max(1.0 - math.exp(-pressure / 2000.0), 0.0), 1.0)
        col = np.asarray(ucol, np.float64) * (1.0 - coef) + np.array([1.0, 0.0, 0.0, 1.0]) * coef
        s = min(max((dist - 5.0) / (4.0 - 5.0), 0.0), 1.0)
        col[3] *= 1.0 - s * s * (3.0 - 2.0 * s)
        if col[3] == 0.0:
            continue
        r2 = float(right @ right)
        corners = [c + up - right, c + up + right, c - up - right, c - up + right]
        clip = [P @ np.append(v, 1.0) for v in corners]
        win = [np.array([(q[0] / q[3] * 0.5 + 0.5) * width, (q[1] / q[3] * 0.5 + 0.5) * height,
                         q[2] / q[3] * 0.5 + 0.5]) for q in clip]
        for tri in ((0, 1, 2), (2, 1, 3)):
            a, b, d = (win[k] for k in tri)
            area = (b[0] - a[0]) * (d[1] - a[1]) - (b[1] - a[1]) * (d[0] - a[0])
            if area == 0.0:
                continue
            x0 = max(int(math.floor(min(a[0], b[0], d[0]))), 0)
            x1 = min(int(math.ceil(max(a[0], b[0], d[0]))), width - 1)
            y0 = max(int(math.floor(min(a[1], b[1], d[1]))), 0)
            y1 = min(int(math.ceil(max(a[1], b[1], d[1]))), height - 1)
            if x0 > x1 or y0 > y1:
                continue
            ys, xs = np.mgrid[y0:y1 + 1, x0:x1 + 1]
            px, py = xs.ravel() + 0.5, ys.ravel() + 0.5
            l0 = ((b[0] - px) * (d[1] - py) - (b[1] - py) * (d[0] - px)) / area
            l1 = ((d[0] - px) * (a[1] - py) - (d[1] - py) * (a[0] - px)) / area
            l2 = 1.0 - l0 - l1
            inside = (l0 >= 0) & (l1 >= 0) & (l2 >= 0)
            lam = np.stack([l0, l1, l2], 1)[inside]
            if not len(lam):
                continue
            w = np.array([clip[k][3] for k in tri])
            verts = np.stack([corners[k] for k in tri])
            persp = lam / w
            fpos = (persp @ verts) / persp.sum(1, keepdims=True)
            depth = lam @ np.array([win[k][2] for k in tri])
            d2 = ((fpos - c) ** 2).sum(1)
            zn = depth * 2.0 - 1.0
            for x, y, dd, m, z in zip(xs.ravel()[inside], ys.ravel()[inside], depth, d2 - r2, zn):
                if -1.0 <= z < 1.0:
                    frags[y * width + x].append((dd, draw, col, m / r2))
    covered = np.zeros(width * height, bool)
    rgba = np.zeros((width * height, 4))
    depth = np.ones(width * height)
    ambiguous = np.zeros(width * height, bool)
    for i, fl in enumerate(frags):
        if not fl:
            continue
        # a strip's two triangles share an edge: one fragment per draw
        best = {}
        for f in fl:
            if f[1] not in best:
                best[f[1]] = f
        fl = list(best.values())
        ambiguous[i] = any(abs(f[3]) <= EDGE_REL for f in fl)
        cov = sorted((f for f in fl if f[3] <= 0.0), key=lambda f: (f[0], f[1]))
        if not cov:
            continue
        covered[i] = True
        rgba[i] = cov[0][2]
        depth[i] = cov[0][0]
        if len(cov) > 1 and cov[1][0] - cov[0][0] <= DEPTH_TIE:
            ambiguous[i] = True
    shape = (height, width)
    return covered.reshape(shape), rgba.reshape(shape + (4,)), depth.reshape(shape), ambiguous.reshape(shape)


def _random_camera(rng, lo, hi, width, height):
    centre = (lo + hi) / 2.0
    radius = float(np.linalg.norm(hi - lo)) / 2.0
    direction = rng.normal(size=3)
    direction /= np.linalg.norm(direction)
    eye = centre + direction * rng.uniform(2.5, 4.0) * radius
    fov = math.radians(rng.uniform(30.0, 70.0))
    return render.perspective(fov, width / height, 0.05, 60.0), render.look_at(eye, centre)


def test_oracle_matches_an_independent_float64_rasteriser():
    """Random particles (positions, pressures, sizes, colours) under random
    cameras, both layers: the C oracle (float32, per-pixel plane solve)
    against the float64 GL-pipeline restatement above.  Outside the
    ambiguous pixels coverage is identical, RGBA8 within 1 step per
    channel and window depth within 5e-7."""
    rng = np.random.default_rng(2024)
    width, height = 160, 120
    compared = 0
    for trial in range(6):
        n, s = int(rng.integers(80, 200)), int(rng.integers(0, 60))
        dyn = np.zeros((n, 4), np.float32)
        dyn[:, :3] = rng.uniform(-2.0, 2.0, size=(n, 3))
        dyn[:, 3] = rng.choice([0.0, 1.0], size=n) * rng.uniform(-500.0, 8000.0, size=n)
        stat = rng.uniform(-2.0, 2.0, size=(s, 3)).astype(np.float32)
        lo = np.minimum(dyn[:, :3].min(0), stat.min(0) if s else dyn[:, :3].min(0)).astype(np.float64)
        hi = np.maximum(dyn[:, :3].max(0), stat.max(0) if s else dyn[:, :3].max(0)).astype(np.float64)
        proj, view = _random_camera(rng, lo, hi, width, height)
        model = render.identity() if trial % 2 == 0 else np.ascontiguousarray(
            (np.diag([1.5, 1.5, 1.5, 1.0]).T.reshape(16)), np.float32)
        dyn_layer = (float(rng.uniform(0.1, 0.6)), tuple(rng.uniform(0.0, 1.0, size=4)))
        stat_layer = (float(rng.uniform(0.1, 0.4)), tuple(rng.uniform(0.0, 1.0, size=4))) if s else None
        rgba, depth = oracle_splat(proj, view, model, width, height, dyn, dyn_layer, stat, stat_layer)
        cov64, rgba64, depth64, amb = splat_f64(proj, view, model, width, height, dyn, dyn_layer, stat,
                                                stat_layer)
        ok = ~amb
        assert amb.mean() < 0.05, amb.mean()
        assert cov64[ok].sum() > 200, cov64[ok].sum()
        covered32 = depth < 1.0
        assert np.array_equal(covered32[ok], cov64[ok])
        both = ok & cov64
        want = np.floor(np.clip(rgba64[both], 0.0, 1.0) * 255.0 + 0.5)
        assert np.abs(rgba[both].astype(np.int64) - want).max() <= COLOUR_TOL
        assert np.abs(depth[both].astype(np.float64) - depth64[both]).max() <= DEPTH_TOL
        compared += int(ok.sum())
    assert compared > 6 * width * height * 0.9
