"""Emitters, rain and Drop (the host side of App::UpdateEmitter and
cSPH::Drop) against the NumPy restatement (oracle/emit.py) and, for the
scene fields, the reference's own loader (tests/golden/scenes.npz)."""
import os

import numpy as np
import pytest

from oracle import emit as oemit
from pibiti_gb300.sph import Scene

REF_SCENES = os.path.join(os.environ.get("PIBITI_REFERENCE_ROOT", "/root/reference"), "Scenes.xml")
# rot.z of an emitter is never initialised nor used by the reference
KEEP = np.ones(38, bool)
KEEP[[5, 14, 23, 32]] = False


def _motion(s):
    m = s.motion
    out = []
    for e in m.emit:
        out += [e.pos.x, e.pos.y, e.pos.z, e.rot.x, e.rot.y, e.rot.z, e.vel, e.size, e.size2]
    return np.array(out + [m.rVel, m.r2Vel], np.float32)


def test_motion_matches_reference(golden):
    g = golden("scenes.npz")
    for xml, ref in zip(g["xml"], g["motion"]):
        np.testing.assert_array_equal(_motion(Scene.parse(str(xml)))[KEEP], ref[KEEP], err_msg=str(xml)[:80])


def test_motion_of_reference_file(golden):
    if not os.path.exists(REF_SCENES):
        pytest.skip("reference Scenes.xml not present")
    g = golden("scenes.npz")
    for i in range(Scene.count(REF_SCENES)):
        np.testing.assert_array_equal(_motion(Scene.load(REF_SCENES, i))[KEEP], g["file_motion"][i][KEEP])


@pytest.mark.parametrize("size,size2,rot", [(4, 0, (0, 0)), (4, 3, (30, -45)), (1, 0, (90, 10)),
                                            (10, 2, (-60, 200))])
def test_emitter_particles(size, size2, rot):
    s = Scene.parse(f'<Scene EmitSize="{size}" EmitSize2="{size2}" EmitPos="0.1 0.2 -0.3" '
                    f'EmitVel="2.5" EmitRot="{rot[0]} {rot[1]}" />')
    pos, vel = s.emitter_particles(0)
    e = s.motion.emit[0]
    rp, rv = oemit.emitter((e.pos.x, e.pos.y, e.pos.z), (e.rot.x, e.rot.y), e.vel, e.size, e.size2,
                           s.info.spacing)
    assert len(pos) == len(rp) == size * (size2 or size)
    np.testing.assert_allclose(pos[:, :3], rp, rtol=0, atol=1e-6)
    np.testing.assert_allclose(vel[:, :3], rv, rtol=0, atol=1e-6)
    assert np.all(pos[:, 3] == 0) and np.all(vel[:, 3] == 0)


def test_emitter_off():
    pos, vel = Scene.default().emitter_particles(0)
    assert len(pos) == 0 and len(vel) == 0


@pytest.mark.parametrize("r", [1.0, 2.5, 3.5])
def test_drop_ball(r):
    s = Scene.parse(f'<Scene dropR="{r}" />')
    pos, vel = s.drop_particles()
    p = s.params
    ref = oemit.drop((p.worldMinD.x, p.worldMinD.y, p.worldMinD.z),
                     (p.worldSizeD.x, p.worldSizeD.y, p.worldSizeD.z), r, s.info.spacing)
    assert len(pos) == len(ref)
    np.testing.assert_allclose(pos[:, :3], ref, rtol=0, atol=1e-6)
    assert np.all(vel == 0) and np.all(pos[:, 3] == 1)


def test_drop_capacity_and_random():
    s = Scene.parse('<Scene dropR="2.5" />')
    full, _ = s.drop_particles()
    part, _ = s.drop_particles(capacity=10)
    np.testing.assert_array_equal(part, full[:10])
    a, _ = s.drop_particles(random=True, seed=5)
    b, _ = s.drop_particles(random=True, seed=5)
    c, _ = s.drop_particles(random=True, seed=6)
    np.testing.assert_array_equal(a, b)
    assert len(a) == len(full) and not np.array_equal(a, c)
    p = s.params
    assert np.all(a[:, :3] >= np.array([p.worldMin.x, p.worldMin.y, p.worldMin.z]) - 1e-6)
    assert np.all(a[:, :3] <= np.array([p.worldMax.x, p.worldMax.y, p.worldMax.z]) + 1e-6)


def test_advance_rotor_and_dye():
    s = Scene.parse('<Scene RotorVel="2" Rotor2Vel="-0.5" Rotor2Dist="0.1" />')
    p = s.params
    want = oemit.advance(p.rAngle, p.r2Angle, p.r2Dist, p.dyeClear, s.motion.rVel,
                         s.motion.r2Vel, p.timeStep)
    s.advance()
    assert p.rAngle == pytest.approx(want[0], rel=1e-6)
    assert p.r2Angle == pytest.approx(want[1], rel=1e-6)
    assert p.r2twist == want[2] and p.dyeClear == want[3]
