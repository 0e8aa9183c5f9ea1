"""Checkpoint files (pibiti_gb300.sph write_snapshot / read_snapshot) on the
CPU: parameters byte for byte, arrays, step and the caller's extra arrays
survive the round trip; inconsistent files are refused."""
import numpy as np
import pytest

from pibiti_gb300 import configs
from pibiti_gb300.sph import Scene, read_snapshot, write_snapshot


def _scenes():
    ws = [configs.dambreak_small(side=s, seed=i) for i, s in enumerate((8, 10))]
    ps = [Scene.parse(w.xml).params for w in ws]
    ps[1].stiffness = 4.5
    offs = [0, ws[0].n, ws[0].n + ws[1].n]
    pos = np.concatenate([w.pos for w in ws])
    vel = np.random.default_rng(0).normal(size=pos.shape).astype(np.float32)
    return ps, offs, pos, vel


def test_round_trip(tmp_path):
    ps, offs, pos, vel = _scenes()
    path = str(tmp_path / "s.npz")
    write_snapshot(path, ps, offs, pos, vel, step=123, extra={"dye": np.arange(5, dtype=np.float32),
                                                              "emit_id": np.int64(77)})
    d = read_snapshot(path)
    assert [p.to_bytes() for p in d["params"]] == [p.to_bytes() for p in ps]
    assert d["offsets"] == offs and d["step"] == 123
    np.testing.assert_array_equal(d["pos"], pos)
    np.testing.assert_array_equal(d["vel"], vel)
    np.testing.assert_array_equal(d["extra"]["dye"], np.arange(5, dtype=np.float32))
    assert int(d["extra"]["emit_id"]) == 77


def test_inconsistent_files_refused(tmp_path):
    ps, offs, pos, vel = _scenes()
    path = str(tmp_path / "s.npz")
    write_snapshot(path, ps, offs, pos[:-1], vel[:-1])
    with pytest.raises(ValueError, match="particle count"):
        read_snapshot(path)
    with np.load(str(tmp_path / "s.npz")) as d:
        items = {k: d[k] for k in d.files}
    items["version"] = np.int64(99)
    np.savez(path, **items)
    with pytest.raises(ValueError, match="version"):
        read_snapshot(path)


def test_object_extras_refused(tmp_path):
    ps, offs, pos, vel = _scenes()
    with pytest.raises(TypeError, match="numeric"):
        write_snapshot(str(tmp_path / "s.npz"), ps, offs, pos, vel, extra={"bad": [object()]})
