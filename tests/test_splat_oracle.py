"""The CPU restatement of the headless particle splat (oracle/sph_splat.c),
checked against the shader arithmetic it restates (particle.vert:67-117,
particle.frag:17-22) on hand-computable cases: the disc's size on screen,
the pressure colour, the distance fade and the depth test."""
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
