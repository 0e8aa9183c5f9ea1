"""python -m pibiti_gb300 on the CPU: the scene listing, and the run
command's argument errors (caught before any GPU work)."""
import pytest

from pibiti_gb300 import configs
from pibiti_gb300.__main__ import main, scene_index


@pytest.fixture
def scenes_file(tmp_path):
    a = configs.dambreak_small(side=8).xml.replace("<Scene ", '<Scene name="small A" ')
    b = configs.dambreak_small(side=10).xml.replace("<Scene ", '<Scene name="small B" ')
    p = tmp_path / "Scenes.xml"
    p.write_text(f"<SPH>\n{a}\n{b}\n</SPH>\n")
    return str(p)


def test_scene_listing(scenes_file, capsys):
    assert main(["scenes", scenes_file]) == 0
    lines = capsys.readouterr().out.splitlines()
    assert len(lines) == 2
    assert lines[0].split()[:3] == ["0", "*", "512"] and lines[0].endswith("small A")
    assert lines[1].split()[:2] == ["1", "1000"] and lines[1].endswith("small B")


def test_scene_index(scenes_file):
    assert scene_index(scenes_file, None) == 0
    assert scene_index(scenes_file, "1") == 1
    assert scene_index(scenes_file, "small B") == 1
    with pytest.raises(SystemExit, match="no scene titled"):
        scene_index(scenes_file, "missing")
    with pytest.raises(SystemExit, match="outside"):
        scene_index(scenes_file, "2")


def test_run_needs_a_scene_source():
    with pytest.raises(SystemExit, match="--resume"):
        main(["run"])
