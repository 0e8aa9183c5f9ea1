"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference's own kernels, radix sort and scene loader run on the CPU
through oracle/_ref/libref_emu.so (built by oracle/ref_emu/build_ref.sh from
the reference tree; see oracle/ref.py).  This script needs that tree and is
run by hand:

    PYTHONPATH=. python tests/golden/make_golden.py

It writes
  scenes.npz        SimParams bytes the reference's loader derives for a set
                    of scene elements (their XML text is stored alongside, so
                    the product loader can be checked anywhere), plus the
                    bytes for every scene of the reference's Scenes.xml
  step_<case>.npz   inputs and every stage output of one cSPH::Update
  integrate_<case>.npz  boundary/integrate outputs for boundary types
All inputs are synthetic and seeded.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import oracle.ref as ref  # noqa: E402
from pibiti_gb300 import configs  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SCENES_XML = os.path.join(ref.REF_ROOT, "Scenes.xml")

# Scene elements written for these fixtures: they exercise the attribute map
# (aliases, overrides, base-0 integers, children) of Scene_Load.cpp.
EXTRA_SCENES = [
    '<Scene name="defaults only" />',
    '<Scene World="0.6 0.5 0.6" InitMin="0.1 -0.25 0.1" InitMax="0.3 0.25 0.3" Stiffness="4" />',
    '<Scene World="1.0 0.5 0.16" Init="0.2 0.5 0.16" ParticlesK="32" spacing="1.43" '
    'TimeStep="0.0007" Stiffness="45" bndStiff="90000" Particles="5000" />',
    '<Scene bndType="0x1" bndEffZ="02" HmapType="0" RotorAngle="30" Rotor2Angle="-15" '
    'RotorTwist="0.5" WaveSpeed="2" WaveAmpl="0.01" HSlope="0.2" Hheight="0.3" Hscale="0.05" '
    'HxFq="2" HxOfs="10" HzFq="3" HzOfs="20" HholeR="0.5" />',
    '<Scene ColliderR="0.06" ColliderPos="-0.16 -0.24 0.0" spring="100" damping="0.05" '
    'shear="0.2" maxParInCell="8" minDist="0.8" minDens="0.9" particleR="0.005" '
    'particleH="0.012" CellSize="0.012" RestDensity="998" Viscosity="0.8" Gravity="0 -9.8 0.5" '
    'globalDamping="0.999" distBndSoft="6" distBndHard="0.5" bndDamp="200" bndDampC="50">'
    '<Accel type="1" pos="0 -0.2 0" size="0.02 0.03 0.02" acc="0 20 0" />'
    '<Accel type="2" pos="0.1 -0.1 0" size="0.03 0.05 0.03" acc="5 0 0" />'
    '<Accel type="3" pos="-0.1 0 0.05" size="0.04 0.05 0.06" acc="0 0 -8" />'
    '</Scene>',
    '<Scene PumpAngOut="0.3" PumpHClose="-0.02" PumpRadIn="0.5" ExitVel="0.05" ExitDist="0.03" '
    's1="0.8" s2="0.85" s3="1.1" s4="0.7" s5="0.9" s6="0.8" RotorSizes="1 5 10" RotorType="0" '
    'Rotor2Dist="0.1" colParR="2.5" colParSpc="0.6" RotorBlades="3" />',
    '<Scene EmitSize="4" EmitPos="0.1 0.2 -0.1" EmitVel="2.5" EmitSize2="3" EmitRot="30 -45" '
    'RotorVel="1.5" Rotor2Vel="-0.5" dropR="3.5" rain="20" spacing="1.2" />',
    '<Scene EmitSize="5" EmitPos="0.3 0.3 0.3"><Emitter size="3" pos="0 0.1 0" vel="1" rot="10 20" />'
    '<Emitter size="2" size2="6" pos="-0.2 0 0.1" rot="-90 180" /></Scene>',
]


def _param_bytes(p) -> np.ndarray:
    return np.frombuffer(p.to_bytes(), np.uint8).copy()


def ref_scene_from_xml(xml: str):
    with tempfile.NamedTemporaryFile("w", suffix=".xml", delete=False) as f:
        f.write("<SPH>" + xml + "</SPH>")
        path = f.name
    try:
        return ref.scene_load(path, 0)
    finally:
        os.unlink(path)


def ref_motion_from_xml(xml: str):
    with tempfile.NamedTemporaryFile("w", suffix=".xml", delete=False) as f:
        f.write("<SPH>" + xml + "</SPH>")
        path = f.name
    try:
        return ref.scene_motion(path, 0)
    finally:
        os.unlink(path)


def make_scenes():
    xmls = list(EXTRA_SCENES)
    xmls += [configs.dambreak_small(side=16).xml, configs.dambreak_small(side=32).xml,
             configs.dambreak_double().xml]
    params, extras, motion = [], [], []
    for x in xmls:
        p, ex = ref_scene_from_xml(x)
        params.append(_param_bytes(p))
        extras.append(np.array(ex, np.float32))
        motion.append(ref_motion_from_xml(x))
    n = ref.scene_count(SCENES_XML)
    file_params = np.stack([_param_bytes(ref.scene_load(SCENES_XML, i)[0]) for i in range(n)])
    file_extras = np.stack([np.array(ref.scene_load(SCENES_XML, i)[1], np.float32) for i in range(n)])
    file_motion = np.stack([ref.scene_motion(SCENES_XML, i) for i in range(n)])
    np.savez_compressed(os.path.join(OUT, "scenes.npz"), xml=np.array(xmls), params=np.stack(params),
                        extras=np.stack(extras), motion=np.stack(motion), file_params=file_params,
                        file_extras=file_extras, file_motion=file_motion)
    print(f"scenes.npz: {len(xmls)} scene elements, {n} scenes of Scenes.xml")


def save_step(name, params, pos, vel, note):
    out = ref.update(params, pos, vel)
    np.savez_compressed(os.path.join(OUT, f"step_{name}.npz"), params=_param_bytes(params),
                        pos_in=pos, vel_in=vel, note=np.array(note), **out)
    print(f"step_{name}.npz: N={len(pos)} cells={params.numCells} ({note})")


def make_steps():
    # A: the dam-break block of the 32,768-particle workload at 16^3, in motion
    w = configs.dambreak_small(side=16)
    p, _ = ref_scene_from_xml(w.xml)
    pos, vel = oracle.step(p, w.pos, w.vel, steps=150)
    save_step("dambreak", p, pos, vel, "16^3 dam break after 150 steps")

    # B: same state, maxParInCell=3, so the walk truncates cells (Kernel_Cell.cui:151,245)
    p3 = p.copy()
    p3.maxParInCell = 3
    save_step("truncate", p3, pos, vel, "maxParInCell=3 truncation")

    # C: the reference's default scene (cell smaller than h, collider inside the
    #    box at the -77 sentinel position), accelerators, colour and dye
    xml = ('<Scene Particles="4096" dyeType="1" dyeClear="0" dyeFade="2">'
           '<Accel type="1" pos="0 -0.15 0" size="0.05 0.05 0.05" acc="0 20 0" />'
           '<Accel type="2" pos="0.05 -0.1 0" size="0.04 0.05 0.04" acc="3 0 0" />'
           '<Accel type="3" pos="-0.05 -0.1 0.05" size="0.05 0.06 0.08" acc="0 0 -6" />'
           '</Scene>')
    pc, _ = ref_scene_from_xml(xml)
    pc.dyePos.x, pc.dyePos.y, pc.dyePos.z = 0.0, -0.18, 0.0
    pc.dyeSize.x, pc.dyeSize.y, pc.dyeSize.z = 0.05, 0.05, 0.05
    rng = np.random.default_rng(7)
    n = 4096
    wmin = np.array([pc.worldMin.x, pc.worldMin.y, pc.worldMin.z])
    wmax = np.array([pc.worldMax.x, pc.worldMax.y, pc.worldMax.z])
    # a block in the lower part of the box, around the collider
    lo = wmin + 0.02
    hi = np.array([wmax[0] - 0.02, wmin[1] + 0.12, wmax[2] - 0.02])
    posc = np.ones((n, 4), np.float32)
    posc[:, :3] = rng.uniform(lo, hi, size=(n, 3))
    velc = np.zeros((n, 4), np.float32)
    velc[:, :3] = rng.normal(0, 0.3, size=(n, 3))
    posc, velc = oracle.step(pc, posc, velc, steps=20)
    save_step("features", pc, posc, velc, "default scene, collider, accelerators, colour, dye")

    # C2: the same state with the CLR_Vel colour (the foam estimate and its
    #     second neighbour walk, System.cu:425-498); clrType is not an XML
    #     attribute, so it is set on the parameters
    pf = pc.copy()
    pf.clrType = 3
    save_step("foam", pf, posc, velc, "CLR_Vel foam colour with dye")

    # C3: the CLR_Vel colour at the grid's edges: cell 0 empty with particles
    #     around it (its walk fetches a zero hash that matches cell 0), and
    #     particles in the last x column, whose +x neighbours wrap to the
    #     first cells of the next row (calcGridHash), which are occupied.
    #     Soft walls off, so that one step keeps the particles in their cells
    #     (the hard clamp is half a cell from the wall).
    rng = np.random.default_rng(13)
    pf = pf.copy()
    pf.distBndSoft = 0.0
    cs_ = np.array([pf.cellSize.x, pf.cellSize.y, pf.cellSize.z])
    gx = int(pf.gridSize.x)

    def in_cells(cells, k):
        cells = np.asarray(cells, float)
        c = cells[rng.integers(0, len(cells), k)]
        lo = np.where(c == 0, 0.6, np.where(c == gx - 1, 0.05, 0.3))
        hi = np.where(c == 0, 0.9, np.where(c == gx - 1, 0.35, 0.7))
        return wmin + (c + rng.uniform(lo, hi)) * cs_

    low = [(x, y, z) for x in (0, 1) for y in (0, 1) for z in (0, 1) if (x, y, z) != (0, 0, 0)]
    edge = [(gx - 1, 0, z) for z in (0, 1)]
    pe = np.ones((1024, 4), np.float32)
    pe[:, :3] = np.concatenate([in_cells(low, 768), in_cells(edge, 256)])
    ve = np.zeros((1024, 4), np.float32)
    ve[:, :3] = rng.normal(0, 0.3, (1024, 3))
    save_step("foam_edges", pf, pe, ve, "CLR_Vel foam: empty cell 0, wrapped neighbour cells")

    # C4: ten particles, all in cell 0 (fewer than maxParInCell): the walk of
    #     cell 0 runs past the last particle, where fetches return hash 0
    pt = np.ones((10, 4), np.float32)
    pt[:, :3] = wmin + rng.uniform(0.6, 0.7, (10, 3)) * cs_
    vt = np.zeros((10, 4), np.float32)
    vt[:, :3] = rng.normal(0, 0.02, (10, 3))
    assert pf.maxParInCell > 10
    save_step("foam_tiny", pf, pt, vt, "CLR_Vel foam: all particles in cell 0")

    # D: a grid of more than 65536 cells: 32-bit sort passes
    wd = configs.dambreak_small(side=8)
    xmld = configs.scene_xml(**configs.dambreak_attrs(1024, (0.0, 0.0, 0.0), (2.2, 2.0, 2.2)))
    pd, _ = ref_scene_from_xml(xmld)
    rng = np.random.default_rng(11)
    posd = np.ones((1024, 4), np.float32)
    posd[:, :3] = rng.uniform([0.15, 0.15, 0.15], [2.05, 1.85, 2.05], size=(1024, 3))
    veld = np.zeros((1024, 4), np.float32)
    veld[:, :3] = rng.normal(0, 0.5, size=(1024, 3))
    assert pd.numCells >= 65536, pd.numCells
    save_step("bigrid", pd, posd, veld, f"{pd.numCells} cells, 32-bit sort")
    del wd

    # F-I: the rotor/propeller and height-map colliders (System.cu:253-372)
    rng = np.random.default_rng(21)
    for name, attrs in (("rotor", 'RotorType="1" RotorAngle="20" RotorTwist="0.3"'),
                        ("propeller", 'RotorType="3" RotorSizes="0 3 8" Rotor2Dist="0.12" '
                                      'Rotor2Angle="40" RotorBlades="3"'),
                        ("hmapxz", 'HmapType="1" Hheight="0.02" Hscale="0.05" HxFq="2" HzFq="3" '
                                   'HholeR="-2"'),
                        ("hmapyz", 'HmapType="2" Hheight="0.02" Hscale="0.05" HxFq="2" HzFq="3" '
                                   'HholeR="0.2"')):
        pr, _ = ref_scene_from_xml(f'<Scene Particles="2048" {attrs} />')
        wmin = np.array([pr.worldMin.x, pr.worldMin.y, pr.worldMin.z])
        wmax = np.array([pr.worldMax.x, pr.worldMax.y, pr.worldMax.z])
        pos = np.ones((2048, 4), np.float32)
        if name in ("rotor", "propeller"):  # around the rotor axis position
            c = np.array([pr.collPos.x, pr.collPos.y, pr.collPos.z])
            pos[:, :3] = np.clip(c + rng.normal(0, 0.03, size=(2048, 3)), wmin + 0.01, wmax - 0.01)
        else:
            pos[:, :3] = rng.uniform(wmin + 0.01, wmax - 0.01, size=(2048, 3))
        vel = np.zeros((2048, 4), np.float32)
        vel[:, :3] = rng.normal(0, 0.2, size=(2048, 3))
        save_step(name, pr, pos, vel, f"collider: {attrs}")

    # E: fewer particles than one block
    w = configs.dambreak_small(side=4)
    p4, _ = ref_scene_from_xml(configs.scene_xml(**configs.dambreak_attrs(64, (0, 0, 0), (1, 1, 1))))
    save_step("tiny", p4, w.pos, w.vel, "64 particles")


def make_integrate():
    base, _ = ref_scene_from_xml('<Scene Particles="512" World="0.4 0.5 0.4" />')
    rng = np.random.default_rng(3)
    cases = {
        "box": dict(bndType=0, bndEffZ=0),
        "cyl_y": dict(bndType=1, bndEffZ=0),
        "cyl_z": dict(bndType=2, bndEffZ=0),
        "cyl_yz": dict(bndType=3, bndEffZ=0),
        "sphere": dict(bndType=4, bndEffZ=0),
        "wrap": dict(bndType=0, bndEffZ=1),
        "cycle": dict(bndType=0, bndEffZ=2),
        "wave": dict(bndType=0, bndEffZ=3, r2Angle=0.2, rTwist=0.01, rAngle=0.7),
        "pump": dict(bndType=5, bndEffZ=0),
        "pump_s": dict(bndType=5, bndEffZ=0, angOut=0.7),
    }
    arrays = {}
    for name, kv in cases.items():
        p = base.copy()
        for k, v in kv.items():
            setattr(p, k, v)
        n = 512
        wmin = np.array([p.worldMin.x, p.worldMin.y, p.worldMin.z])
        wmax = np.array([p.worldMax.x, p.worldMax.y, p.worldMax.z])
        pos = np.ones((n, 4), np.float32)
        pos[:, :3] = rng.uniform(wmin - 0.01, wmax + 0.01, size=(n, 3))
        vel = np.zeros((n, 4), np.float32)
        vel[:, :3] = rng.normal(0, 0.5, size=(n, 3))
        vel[:, 3] = rng.uniform(0, 1, size=n)
        npos, nvel = ref.integrate(p, pos, vel)
        arrays[f"{name}_params"] = _param_bytes(p)
        arrays[f"{name}_pos_in"] = pos
        arrays[f"{name}_vel_in"] = vel
        arrays[f"{name}_pos"] = npos
        arrays[f"{name}_vel"] = nvel
    np.savez_compressed(os.path.join(OUT, "integrate.npz"), cases=np.array(list(cases)), **arrays)
    print(f"integrate.npz: {len(cases)} boundary cases")


if __name__ == "__main__":
    if not ref.available():
        sys.exit("the reference tree is needed to generate the golden fixtures")
    make_scenes()
    make_steps()
    make_integrate()
