"""Command line: the scenes of a Scenes.xml file, and one of them stepped.

    python -m pibiti_gb300 scenes Scenes.xml
    python -m pibiti_gb300 run Scenes.xml --scene 3 --steps 1000 --seed 42 --snapshot s.npz
    python -m pibiti_gb300 run Scenes.xml --scene "box small default" --motion
    python -m pibiti_gb300 run --resume s.npz --steps 1000

``scenes`` lists index, particle count and title (``*`` marks the file's
default scene, cSPH::LoadScenes' choice).  ``run`` resets the scene as
cSPH::Reset does (the scene's init type unless --init, seed --seed), steps it
on the GPU and prints one JSON line (wall time including the final readback,
kinetic energy, mean density, largest density deviation, non-finite count,
status flags); --motion applies the per-frame parameter updates of
App::UpdateEmitter (rotor angles, dye clear) before every step; --snapshot
writes a checkpoint that --resume continues.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

from .sph import ARRAY_POS, ARRAY_VEL, SPH, Scene


def scene_index(path: str, scene) -> int:
    """The index of `scene` (an index, or a title) in the file; the file's
    default scene when None."""
    if scene is None:
        return Scene.default_index(path)
    try:
        i = int(scene)
    except ValueError:
        titles = [s.title for s in Scene.load_all(path)]
        if scene not in titles:
            raise SystemExit(f"no scene titled {scene!r} in {path}")
        return titles.index(scene)
    n = Scene.count(path)
    if not 0 <= i < n:
        raise SystemExit(f"scene index {i} outside 0..{n - 1} of {path}")
    return i


def cmd_scenes(args) -> int:
    n = Scene.count(args.file)
    default = Scene.default_index(args.file)
    for i in range(n):
        s = Scene.load(args.file, i)
        print(f"{i:4d} {'*' if i == default else ' '} {s.params.numParticles:10d}  {s.title}")
    return 0


def cmd_run(args) -> int:
    scene, step0, title = None, 0, "(snapshot)"
    if args.resume:
        s, step0, _ = SPH.restore(args.resume)
    else:
        if not args.file:
            raise SystemExit("run: a Scenes.xml file or --resume is needed")
        i = scene_index(args.file, args.scene)
        scene = Scene.load(args.file, i)
        title = scene.title
        kind = scene.info.initType if args.init is None else args.init
        pos, vel = scene.reset(kind, args.seed)
        s = SPH(scene.params)
        s.set_array(ARRAY_POS, pos)
        s.set_array(ARRAY_VEL, vel)
    with s:
        t0 = time.perf_counter()
        if args.motion and scene is not None:
            for _ in range(args.steps):
                scene.advance()
                s.set_params(scene.params)
                s.update(1)
        else:
            s.update(args.steps)
        st = s.stats()[0]
        wall = time.perf_counter() - t0
        if args.snapshot:
            s.snapshot(args.snapshot, step=step0 + args.steps)
        print(json.dumps({"scene": title, "particles": s.n, "steps": args.steps, "step": step0 + args.steps,
                          "wall_s": wall, "particle_steps_per_s": s.n * args.steps / wall if wall > 0 else None,
                          "kinetic_energy": float(st[0]), "mean_density": float(st[1]),
                          "max_density_dev": float(st[2]), "nonfinite": float(st[3]), "flags": s.flags(),
                          "snapshot": args.snapshot}))
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m pibiti_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("scenes", help="list the scenes of a Scenes.xml file")
    a.add_argument("file")
    a.set_defaults(fn=cmd_scenes)
    r = sub.add_parser("run", help="reset a scene and step it on the GPU")
    r.add_argument("file", nargs="?", help="Scenes.xml (not needed with --resume)")
    r.add_argument("--scene", help="index or title (default: the file's default scene)")
    r.add_argument("--steps", type=int, default=1000)
    r.add_argument("--seed", type=int, default=42)
    r.add_argument("--init", type=int, help="reset kind (default: the scene's init type)")
    r.add_argument("--motion", action="store_true", help="per-frame parameter updates before every step")
    r.add_argument("--snapshot", help="checkpoint file written after the steps")
    r.add_argument("--resume", help="checkpoint file to continue from")
    r.set_defaults(fn=cmd_run)
    args = ap.parse_args(argv)
    return args.fn(args)


if __name__ == "__main__":
    sys.exit(main())
