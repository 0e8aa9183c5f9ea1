"""Restatement of the reference's emitter, Drop and per-frame parameter
updates in NumPy (float64), for tests only:

* emitter particles: App::UpdateEmitter (App/Update.cpp:64-91) with the
  OpenGL modelview matrix M = Rx(rot.x) Ry(-rot.y) (glRotatef, degrees,
  right-multiplied onto the identity) applied transposed by App::mulTr
  (App/Input.cpp:587-592);
* Drop: cSPH::Drop (SPH_Init.cpp:83-117), centred variant;
* rotor angles and dye countdown: App/Update.cpp:14-23.
"""
from __future__ import annotations

import numpy as np


def gl_rotate(deg: float, axis: str) -> np.ndarray:
    a = np.deg2rad(deg)
    c, s = np.cos(a), np.sin(a)
    if axis == "x":
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def emitter(pos, rot, vel, size, size2, spacing):
    """(positions (n, 3), velocities (n, 3)) of one frame of one emitter."""
    if size <= 0:
        return np.zeros((0, 3)), np.zeros((0, 3))
    ex, ey = size, (size2 if size2 else size)
    m = gl_rotate(rot[0], "x") @ gl_rotate(-rot[1], "y")
    zx, zy = (ex - 1) * 0.5, (ey - 1) * 0.5
    pts = [((x - zx) * spacing, (y - zy) * spacing, -spacing) for y in range(ey) for x in range(ex)]
    p = np.array(pts) @ m + np.asarray(pos, np.float64)  # row vector times M = (M^T v)^T
    v = np.array([0.0, 0.0, vel]) @ m
    return p, np.tile(v, (len(p), 1))


def drop(world_min_d, world_size_d, drop_r: float, spacing: float):
    """Positions (n, 3) of the centred Drop ball, in the reference's loop order."""
    db = (drop_r + 1.0) * spacing
    c = np.asarray(world_min_d, np.float64) + db + 0.5 * (np.asarray(world_size_d, np.float64) - 2 * db)
    lo = int(-drop_r)
    out = []
    for z in range(lo, int(np.floor(drop_r)) + 1):
        for y in range(lo, int(np.floor(drop_r)) + 1):
            for x in range(lo, int(np.floor(drop_r)) + 1):
                if x * x + y * y + z * z <= drop_r * drop_r:
                    out.append((x * spacing + c[0], y * spacing + c[1], z * spacing + c[2]))
    return np.array(out)


def advance(r_angle, r2_angle, r2_dist, dye_clear, r_vel, r2_vel, dt):
    """One frame of the rotor angles and the dye countdown."""
    r2_twist = None
    if r_vel != 0.0:
        r_angle += r_vel * dt
        if r2_dist > 0.0:
            r2_angle += r_vel * r2_vel * dt
            r2_twist = -1.0 if r2_vel < 0.0 else 1.0
    if dye_clear > 0:
        dye_clear -= 1
    return r_angle, r2_angle, r2_twist, dye_clear
