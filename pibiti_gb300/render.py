"""Headless screen-space fluid rendering (sph_render_*): the reference's
OpenGL fluid pipeline (Graphics/render_particles.cpp and its shaders) as CUDA
passes into device buffers.

    r = Renderer(1280, 720)
    mv = look_at(eye=(0.5, 1.2, 2.5), target=(0.5, 0.3, 0.5))
    pr = perspective(60.0, 1280 / 720, 0.1, 10.0)
    depth, thickness, rgba = r.frame(pos_device, mv, pr, radius=0.02, method=1, iterations=8)
    save_ppm("frame.ppm", rgba.cpu().numpy())

From the command line (the 1,048,576-particle double dam break, from a state
saved by ``bench.py --save-state`` or after --steps steps from the start):

    python -m pibiti_gb300.render --state st.npz --frames 10 --out frame.ppm
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib

MAX_KERNEL_CENTER = 16


class RenderParams(ctypes.Structure):
    _fields_ = [("modelview", ctypes.c_float * 16), ("projection", ctypes.c_float * 16),
                ("point_radius", ctypes.c_float), ("point_scale", ctypes.c_float),
                ("method", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("kernel_center", ctypes.c_int32), ("sigma", ctypes.c_float),
                ("env_color", ctypes.c_float * 3), ("background", ctypes.c_float * 3)]


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """gluLookAt as a column-major 4x4 (float32, flat 16)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m.T.astype(np.float32).ravel()  # column-major


def perspective(fovy_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """gluPerspective as a column-major 4x4 (float32, flat 16)."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = f / aspect, f
    m[2, 2], m[2, 3] = (far + near) / (near - far), 2.0 * far * near / (near - far)
    m[3, 2] = -1.0
    return m.T.astype(np.float32).ravel()


def point_scale(height: int, fovy_deg: float) -> float:
    """ParticleRenderer::updPScale (render_particles.h:39)."""
    return height / math.tan(math.radians(fovy_deg) * 0.5)


class Renderer:
    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self._r = ctypes.c_void_p()
        _lib.check(_lib.lib().sph_render_create(width, height, ctypes.byref(self._r)))

    def close(self) -> None:
        if self._r:
            _lib.lib().sph_render_destroy(self._r)
            self._r = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, modelview, projection, radius: float, scale: float = None, method: int = 0,
               iterations: int = 0, kernel_center: int = 7, sigma: float = 0.01,
               env=(0.6, 0.7, 0.8), background=(0.1, 0.1, 0.12), fovy: float = 60.0) -> RenderParams:
        p = RenderParams()
        p.modelview[:] = [float(v) for v in np.asarray(modelview, np.float32).ravel()]
        p.projection[:] = [float(v) for v in np.asarray(projection, np.float32).ravel()]
        p.point_radius = radius
        p.point_scale = point_scale(self.height, fovy) if scale is None else scale
        p.method, p.iterations, p.kernel_center, p.sigma = method, iterations, kernel_center, sigma
        p.env_color[:] = list(env)
        p.background[:] = list(background)
        return p

    def frame(self, pos, modelview, projection, radius: float, foam=None, **kw):
        """pos: a CUDA tensor of (n, 4) float32.  Returns (depth, thickness,
        rgba) CUDA tensors of (H, W), (H, W), (H, W, 4), row 0 at the bottom.
        foam: the particles' colours ((n, 4) float32 CUDA tensor, the step's
        colour output); when given, the foam overlay is drawn over rgba."""
        p = self.params(modelview, projection, radius, **kw)
        out = self.frame_params(pos, p)
        if foam is not None:
            self.foam_params(pos, foam, p, out[2])
        return out

    def frame_params(self, pos, p: RenderParams):
        import torch
        H, W = self.height, self.width
        depth = torch.empty((H, W), dtype=torch.float32, device="cuda")
        thick = torch.empty((H, W), dtype=torch.float32, device="cuda")
        rgba = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        frags = ctypes.c_uint64()
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        torch.cuda.synchronize()
        _lib.check(_lib.lib().sph_render_frame(self._r, ctypes.c_void_p(ctypes.addressof(p)), vp(pos),
                                               pos.shape[0],
                                               vp(depth), vp(thick), vp(rgba), ctypes.byref(frags)))
        self.fragments = frags.value
        return depth, thick, rgba

    def foam_params(self, pos, color, p: RenderParams, rgba=None):
        """The foam overlay (sph_render_foam): color[:, 0] of each particle
        decides its foam sprites; rgba (an (H, W, 4) CUDA tensor, or None) is
        overwritten where they land.  Returns their depth, (H, W), 1.0 where
        no foam was drawn."""
        import torch
        if tuple(color.shape) != tuple(pos.shape):
            raise ValueError("foam colours must have the positions' shape (n, 4)")
        depth = torch.empty((self.height, self.width), dtype=torch.float32, device="cuda")
        vp = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        torch.cuda.synchronize()
        _lib.check(_lib.lib().sph_render_foam(self._r, ctypes.c_void_p(ctypes.addressof(p)), vp(pos), vp(color),
                                              pos.shape[0], vp(rgba), vp(depth)))
        return depth


def save_ppm(path: str, rgba: np.ndarray) -> None:
    """Writes an (H, W, 4) float image (row 0 at the bottom) as binary PPM."""
    img = np.clip(np.asarray(rgba)[::-1, :, :3], 0.0, 1.0)
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(f"P6 {w} {h} 255\n".encode())
        f.write((img * 255.0 + 0.5).astype(np.uint8).tobytes())


def main(argv=None) -> int:
    """Renders the double dam break: one step with the colour output on (the
    foam overlay's input), then --frames frames (G-buffer, --iterations
    curvature-flow passes, shading) and as many foam overlays, each timed as
    a synchronous call.  Prints one JSON line; --out writes the last frame."""
    import argparse
    import json
    import time

    import torch

    from . import configs
    from .sph import ARRAY_POS, ARRAY_VEL, SPH, Scene
    ap = argparse.ArgumentParser(prog="python -m pibiti_gb300.render")
    ap.add_argument("--state", help="npz with pos and vel (bench.py --save-state)")
    ap.add_argument("--steps", type=int, default=200, help="steps from the start when no --state")
    ap.add_argument("--frames", type=int, default=10)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--iterations", type=int, default=8)
    ap.add_argument("--out", help="PPM file for the last frame")
    args = ap.parse_args(argv)
    w = configs.dambreak_double()
    params = Scene.parse(w.xml).params
    pos0, vel0 = w.pos, w.vel
    if args.state:
        st = np.load(args.state)
        pos0, vel0 = st["pos"], st["vel"]
    with SPH(params) as s:
        s.set_array(ARRAY_POS, pos0)
        s.set_array(ARRAY_VEL, vel0)
        if not args.state and args.steps > 1:
            s.update(args.steps - 1)
        clr = torch.empty((s.n, 4), dtype=torch.float32, device="cuda")
        s.set_color_output(clr)
        s.update(1)
        s.set_color_output(None)
        pos = torch.empty((s.n, 4), dtype=torch.float32, device="cuda")
        s.get_array(ARRAY_POS, out=pos)
    torch.cuda.synchronize()
    W, H = args.width, args.height
    mv = look_at((3.0, 2.6, 6.8), (3.0, 0.6, 0.85))
    pr = perspective(60.0, W / H, 0.1, 20.0)
    frame_s, foam_s = [], []
    with Renderer(W, H) as r:
        prm = r.params(mv, pr, radius=2.0 * params.particleR, method=1, iterations=args.iterations)
        for _ in range(max(args.frames, 1)):
            t0 = time.perf_counter()
            rgba = r.frame_params(pos, prm)[2]
            t1 = time.perf_counter()
            fdepth = r.foam_params(pos, clr, prm, rgba)
            foam_s.append(time.perf_counter() - t1)
            frame_s.append(t1 - t0)
        frags = r.fragments
    if args.out:
        save_ppm(args.out, rgba.cpu().numpy())
    print(json.dumps({"width": W, "height": H, "particles": int(len(pos0)), "frames": len(frame_s),
                      "frame_ms": 1e3 * float(np.median(frame_s)), "foam_ms": 1e3 * float(np.median(foam_s)),
                      "fragments": int(frags), "foam_pixels": int((fdepth < 1).sum().item())}))
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(main())
