"""Headless particle splats on the GPU (sph_engine_render) against the CPU
restatement (oracle/sph_splat.c): every byte of the RGBA image and every
depth value must match, because both evaluate the same rounded operations
(the shader arithmetic of particle.vert and particle.frag, with the same e^x
routine) per pixel and resolve the depth test by (depth, draw index)."""
import math

import numpy as np
import pytest

from oracle_lib import oracle_splat
from sphfluidsimulation_gb300 import render, scenes
from sphfluidsimulation_gb300.engine import SimulationEngineCUDA

pytestmark = pytest.mark.gpu

DYN = (0.1, (1.0, 1.0, 1.0, 1.0))        # the reference application's layers
STAT = (0.03, (0.0, 0.0, 1.0, 1.0))


def both(e, proj, view, model, width, height, dyn=DYN, stat=STAT):
    rgba, depth = e.render(proj, view, model, width, height, dyn, stat)
    d = e.read_dynamic_buffer()
    dyn4 = np.concatenate([d["pos"], d["pressure"][:, None]], 1)
    sp, _ = e.read_static()
    rgba_o, depth_o = oracle_splat(proj, view, model, width, height, dyn4, dyn, sp["pos"], stat)
    return (rgba, depth), (rgba_o, depth_o)


def assert_same_image(g, o, what):
    (rgba, depth), (rgba_o, depth_o) = g, o
    bad = np.nonzero((rgba != rgba_o).any(-1) | (depth.view(np.uint32) != depth_o.view(np.uint32)))
    assert bad[0].size == 0, f"{what}: {bad[0].size} pixels differ, first at {bad[0][0]},{bad[1][0]}"


def test_render_dam_break_matches_oracle():
    sc = scenes.dam_break((20, 12, 20), 0.02, 0.04, (0.6, 0.4, 0.6), 0, mass=0.008, name="dam_4800")
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.update(sc.dt, 30)
    # the box scaled 10x by the model matrix, seen from 9 units away
    model = np.diag([10.0, 10.0, 10.0, 1.0]).astype(np.float32).T.reshape(16)
    view = render.look_at((3.0, 6.0, 11.0), (3.0, 1.0, 3.0))
    proj = render.perspective(math.radians(120.0), 4.0 / 3.0, 0.1, 1000.0)
    g, o = both(e, proj, view, model, 320, 240)
    assert_same_image(g, o, "dam break")
    covered = g[0][..., 3] > 0
    assert covered.sum() > 1000                       # fluid and walls are on screen (discs ~1.5 px wide)
    assert (g[0][covered][:, 2] == 255).any()          # some wall pixels are blue (static layer)


def test_render_close_up_fade_and_ties():
    """Camera inside the fade distance of part of the scene, coincident
    particles (depth ties) and a wide field of view."""
    rng = np.random.default_rng(4)
    pos = rng.uniform(-2.0, 2.0, size=(3000, 3)).astype(np.float32)
    pos[1000:1100] = pos[900:1000]                     # exact duplicates: ties resolved by draw order
    sc = scenes.Scene(name="cloud", dyn_pos=pos, static_pos=np.zeros((0, 3), np.float32),
                      params=scenes.water_params(0.05, 0.1), dt=1e-4, steps=0)
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.update(sc.dt, 2)
    view = render.look_at((0.0, 0.0, 6.5), (0.0, 0.0, 0.0))
    proj = render.perspective(math.radians(120.0), 1.0, 0.1, 1000.0)
    g, o = both(e, proj, view, render.identity(), 200, 200, dyn=(0.3, (0.2, 0.6, 1.0, 1.0)), stat=None)
    assert_same_image(g, o, "close-up")
    alphas = np.unique(g[0][..., 3])
    assert alphas.size > 3                             # faded pixels between 0 and 255


def test_render_config0_after_steps_matches_oracle():
    sc = scenes.config0(steps=0)
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.update(sc.dt, 20)
    model = np.diag([8.0, 8.0, 8.0, 1.0]).astype(np.float32).T.reshape(16)
    view = render.look_at((9.0, 5.0, 12.0), (4.0, 1.0, 2.8))
    proj = render.perspective(math.radians(120.0), 16.0 / 9.0, 0.1, 1000.0)
    g, o = both(e, proj, view, model, 640, 360)
    assert_same_image(g, o, "config 0")
