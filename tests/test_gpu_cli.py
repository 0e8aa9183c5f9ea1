"""python -m pibiti_gb300 run on the GPU: reset, step, checkpoint and resume
through the command line, against the same steps run in one go."""
import json

import pytest

from pibiti_gb300 import configs
from pibiti_gb300.__main__ import main

pytestmark = pytest.mark.gpu


@pytest.fixture
def scenes_file(tmp_path):
    a = configs.dambreak_small(side=8).xml.replace("<Scene ", '<Scene name="small A" ')
    b = configs.dambreak_small(side=10).xml.replace("<Scene ", '<Scene name="small B" ')
    p = tmp_path / "Scenes.xml"
    p.write_text(f"<SPH>\n{a}\n{b}\n</SPH>\n")
    return str(p)


def _run(capsys, argv):
    assert main(argv) == 0
    return json.loads(capsys.readouterr().out.strip().splitlines()[-1])


def test_run_snapshot_resume(cuda, scenes_file, tmp_path, capsys):
    snap = str(tmp_path / "s.npz")
    whole = _run(capsys, ["run", scenes_file, "--scene", "small B", "--steps", "30"])
    first = _run(capsys, ["run", scenes_file, "--scene", "1", "--steps", "20", "--snapshot", snap])
    rest = _run(capsys, ["run", "--resume", snap, "--steps", "10"])
    assert whole["particles"] == first["particles"] == rest["particles"] == 1000
    assert first["step"] == 20 and rest["step"] == 30
    # the plain step keeps no state beyond the checkpoint: the resumed run
    # ends on the same bits as the uninterrupted one
    for k in ("kinetic_energy", "mean_density", "max_density_dev"):
        assert rest[k] == whole[k], k
    assert rest["nonfinite"] == 0 and rest["flags"] == whole["flags"]


def test_run_with_motion(cuda, scenes_file, capsys):
    out = _run(capsys, ["run", scenes_file, "--steps", "10", "--motion"])
    assert out["scene"] == "small A" and out["particles"] == 512 and out["nonfinite"] == 0
    assert out["mean_density"] > 0
