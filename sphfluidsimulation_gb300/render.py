"""Camera matrices and image output for the headless particle renderer
(``SimulationEngineCUDA.render`` / ``sph_engine_render``).

Matrices are 4x4 float32 in OpenGL's column-major layout (element
``[col * 4 + row]``), applied to column vectors, as the reference's shaders
take their ``u_projMatrix``, ``u_viewMatrix`` and ``u_modelMatrix``
uniforms.  The reference's application uses a 120-degree vertical field of
view with planes 0.1 and 1000 (SimulationVisualisationScene.cpp:133).
"""
from __future__ import annotations

import math
from typing import Sequence

import numpy as np


def _colmajor(m: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, np.float64).T.reshape(16), np.float32)


def perspective(fov_y: float, aspect: float, near: float, far: float) -> np.ndarray:
    """The OpenGL perspective projection (view space looks down -z, clip z
    in [-w, w] between the near and far planes)."""
    f = 1.0 / math.tan(fov_y / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[2, 3] = 2.0 * far * near / (near - far)
    m[3, 2] = -1.0
    return _colmajor(m)


def look_at(eye: Sequence[float], target: Sequence[float], up: Sequence[float] = (0.0, 1.0, 0.0)) -> np.ndarray:
    """A view matrix placing the eye at ``eye`` looking at ``target``."""
    e, t, u = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = t - e
    f /= np.linalg.norm(f)
    s = np.cross(f, u)
    s /= np.linalg.norm(s)
    uu = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, uu, -f
    m[:3, 3] = -m[:3, :3] @ e
    return _colmajor(m)


def identity() -> np.ndarray:
    return _colmajor(np.eye(4))


def write_ppm(path: str, rgba: np.ndarray, background: Sequence[int] = (0, 0, 0)) -> None:
    """Writes an RGBA8 render (row 0 at the bottom) as a binary PPM, top row
    first, with alpha composited over ``background``."""
    img = np.asarray(rgba, np.float64)[::-1]
    a = img[..., 3:4] / 255.0
    rgb = img[..., :3] * a + np.asarray(background, np.float64) * (1.0 - a)
    out = np.clip(np.rint(rgb), 0, 255).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(f"P6 {out.shape[1]} {out.shape[0]} 255\n".encode())
        f.write(out.tobytes())
