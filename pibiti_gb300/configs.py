"""Synthetic workloads: scene descriptions and seeded initial particle states.

Each workload is a ``<Scene .../>`` element written with the reference's own
Scenes.xml attribute names (source/SPH/Scene_Load.cpp:186-287), so the same
scene loader that reads Scenes.xml derives its constants, plus a seeded
generator for the initial positions (placed through the particle-buffer API,
like cSPH::setArray, source/SPH/SPH_Util.cpp:59-71).

Dam-break blocks are cubic lattices at spacing s = 0.5 h with +-1 % of s
uniform jitter.  particleR = s * (3 / (4 pi))^(1/3) makes the particle mass
rho0 * 4/3 pi r^3 equal to rho0 * s^3.  Particles are numbered x fastest,
then z, then y, the order cSPH::Reset fills a volume in with InitLast=1
(source/SPH/SPH_Init.cpp:40-48).  The sphere collider is parked far outside
the box (without ColliderPos the loader would place it inside,
Scene.cpp:173-174).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

H_DAMBREAK = 0.0457
SPACING = 0.5 * H_DAMBREAK
R_FROM_S = (3.0 / (4.0 * math.pi)) ** (1.0 / 3.0)


def particle_radius(spacing: float) -> float:
    return spacing * R_FROM_S


def scene_xml(**attrs) -> str:
    def fmt(v):
        if isinstance(v, (tuple, list)):
            return " ".join(repr(float(c)) for c in v)
        return repr(v) if isinstance(v, float) else str(v)
    body = " ".join(f'{k}="{fmt(v)}"' for k, v in attrs.items())
    return f"<Scene {body} />"


def dambreak_attrs(n: int, world_min, world_max, h: float = H_DAMBREAK,
                   spacing: float = SPACING, stiffness: float = 3.0,
                   viscosity: float = 3.5, dt: float = 1e-3, **extra) -> dict:
    a = dict(
        Particles=n, TimeStep=float(dt), Gravity=(0.0, -9.8, 0.0),
        particleR=float(particle_radius(spacing)), particleH=float(h), CellSize=float(h),
        RestDensity=1000.0, Stiffness=float(stiffness), Viscosity=float(viscosity),
        WorldMin=tuple(world_min), WorldMax=tuple(world_max),
        ColliderPos=(-1000.0, -1000.0, -1000.0),
        maxParInCell=16, minDist=1.0, minDens=1.0,
        distBndSoft=8.0, distBndHard=1.0, bndStiff=30000.0, bndDamp=256.0, bndDampC=60.0,
    )
    a.update(extra)
    return a


def lattice(dims, origin, spacing: float, rng: np.random.Generator,
            jitter: float = 0.01) -> np.ndarray:
    """float4 positions of a dims=(nx, ny, nz) block, x fastest then z then y."""
    nx, ny, nz = dims
    iy, iz, ix = np.meshgrid(np.arange(ny), np.arange(nz), np.arange(nx), indexing="ij")
    p = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    p = np.asarray(origin, np.float64) + spacing * p
    p += rng.uniform(-jitter * spacing, jitter * spacing, size=p.shape)
    out = np.ones((len(p), 4), np.float32)
    out[:, :3] = p
    return out


@dataclass
class Workload:
    name: str
    xml: str
    pos: np.ndarray
    vel: np.ndarray
    steps: int
    notes: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.pos)


def _inset(r: float, soft: float = 8.0) -> float:
    # The reference insets the initial volume by (distBndSoft - particleR)
    # from the walls (Scene.cpp:163-164).
    return soft * r - r


def dambreak_small(side: int = 32, seed: int = 42, steps: int = 1000) -> Workload:
    """One side^3 block in the low corner of a unit box (side=32: 32,768
    particles; the smaller sides are the parity cases)."""
    r = particle_radius(SPACING)
    o = _inset(r)
    rng = np.random.default_rng(seed)
    pos = lattice((side, side, side), (o, o + r, o), SPACING, rng)
    n = len(pos)
    xml = scene_xml(**dambreak_attrs(n, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)))
    return Workload(f"dambreak_{n}", xml, pos, np.zeros_like(pos), steps,
                    dict(box=(1.0, 1.0, 1.0), block=(side,) * 3))


def dambreak_double(nx: int = 64, ny: int = 128, nz: int = 64, seed: int = 42,
                    steps: int = 2000, box=(6.0, 3.4, 1.7)) -> Workload:
    """Two nx*ny*nz blocks at the two x ends of the box (defaults: 1,048,576
    particles in a 6.0 x 3.4 x 1.7 m box, 132 x 75 x 38 cells)."""
    r = particle_radius(SPACING)
    o = _inset(r)
    rng = np.random.default_rng(seed)
    a = lattice((nx, ny, nz), (o, o + r, o), SPACING, rng)
    x1 = box[0] - o - (nx - 1) * SPACING
    b = lattice((nx, ny, nz), (x1, o + r, o), SPACING, rng)
    pos = np.concatenate([a, b])
    n = len(pos)
    xml = scene_xml(**dambreak_attrs(n, (0.0, 0.0, 0.0), tuple(box)))
    return Workload(f"double_dambreak_{n}", xml, pos, np.zeros_like(pos), steps,
                    dict(box=tuple(box), block=(nx, ny, nz)))


def uniform_stress(n: int = 16_777_216, seed: int = 42, steps: int = 200,
                   box=(4.0, 1.0, 4.0), fill: float = 0.6, neighbours: float = 40.0) -> Workload:
    """n particles uniform-random in the lower `fill` of the box height, h
    chosen so a sphere of radius h holds `neighbours` particles on average."""
    vol = box[0] * box[1] * fill * box[2]
    density = n / vol
    h = (neighbours / (4.0 / 3.0 * math.pi * density)) ** (1.0 / 3.0)
    spacing = density ** (-1.0 / 3.0)
    r = particle_radius(spacing)
    o = _inset(r)
    rng = np.random.default_rng(seed)
    pos = np.ones((n, 4), np.float32)
    lo = np.array([o, o, o])
    hi = np.array([box[0] - o, box[1] * fill, box[2] - o])
    pos[:, :3] = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    xml = scene_xml(**dambreak_attrs(n, (0.0, 0.0, 0.0), tuple(box), h=h, spacing=spacing))
    return Workload(f"uniform_{n}", xml, pos, np.zeros_like(pos), steps,
                    dict(box=tuple(box), h=h, spacing=spacing))


@dataclass
class Ensemble:
    name: str
    xmls: list
    pos: np.ndarray  # all scenes concatenated, scene order
    vel: np.ndarray
    sizes: list
    steps: int
    notes: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.pos)


def ensemble(scenes: int = 256, nmin: int = 4096, nmax: int = 65536, seed: int = 42,
             steps: int = 500) -> Ensemble:
    """Independent dam-break scenes for the batched ensemble: particle counts
    log-uniform in [nmin, nmax] rounded to 512, stiffness k ~ U[1, 5] and
    viscosity mu ~ U[1, 6] per scene, same h, spacing and dt.  Each scene is a
    16 x 16 (n <= 16384) or 32 x 32 based column filled layer by layer from
    the low corner of a box three columns wide."""
    rng = np.random.default_rng(seed)
    r = particle_radius(SPACING)
    o = _inset(r)
    xmls, pos, sizes = [], [], []
    for s in range(scenes):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        n = max(512, (n + 256) // 512 * 512)
        base = 16 if n <= 16384 else 32
        layers = -(-n // (base * base))
        block = lattice((base, layers, base), (o, o + r, o), SPACING, rng)[:n]
        width = (base - 1) * SPACING + 2 * o
        box = (3.0 * width, (layers - 1) * SPACING * 1.25 + 2 * o + 0.1, width + 0.02)
        k = float(rng.uniform(1.0, 5.0))
        mu = float(rng.uniform(1.0, 6.0))
        xmls.append(scene_xml(**dambreak_attrs(n, (0.0, 0.0, 0.0), box, stiffness=k,
                                               viscosity=mu)))
        pos.append(block)
        sizes.append(n)
    pos = np.concatenate(pos)
    return Ensemble(f"ensemble_{scenes}", xmls, pos, np.zeros_like(pos), sizes, steps,
                    dict(total=int(pos.shape[0])))
