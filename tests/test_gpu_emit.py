"""Emitted and dropped particles written into a running system through the
buffer API (sph_set_array at the running emit index), then stepped."""
import numpy as np
import pytest

from pibiti_gb300 import configs
from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

pytestmark = pytest.mark.gpu


def test_emit_wraps_and_steps(cuda):
    w = configs.dambreak_small(side=8)
    base = Scene.parse(w.xml)
    em = Scene.parse(w.xml.replace("<Scene ", '<Scene EmitSize="5" EmitSize2="4" '
                                   'EmitPos="0.5 0.6 0.5" EmitVel="1.5" EmitRot="20 30" ', 1))
    ep, ev = em.emitter_particles(0)
    assert len(ep) == 20
    with SPH(base.params) as s:
        s.set_array(ARRAY_POS, w.pos)
        s.set_array(ARRAY_VEL, w.vel)
        s.update(2)
        start = s.n - 7  # the block wraps after 7 particles
        nxt = s.emit(ep, ev, start)
        assert nxt == 13
        pos, vel = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL)
        np.testing.assert_array_equal(pos[start:], ep[:7])
        np.testing.assert_array_equal(pos[:13], ep[7:])
        np.testing.assert_array_equal(vel[start:], ev[:7])
        dp, dv = base.drop_particles(capacity=s.n - nxt)
        nxt2 = s.emit(dp, dv, nxt)
        np.testing.assert_array_equal(s.get_array(ARRAY_POS)[nxt:nxt + len(dp)], dp)
        assert nxt2 == (nxt + len(dp)) % s.n
        s.update(5)
        st = s.stats()[0]
        assert st[3] == 0 and np.isfinite(s.get_array(ARRAY_POS)).all()
