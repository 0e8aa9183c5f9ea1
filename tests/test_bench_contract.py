"""bench.py's reference arm on the CPU: one JSON line with our arm's metric,
unit and direction, the oracle port as the CPU implementation, and an e2e
block with no host-device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    sys.path.insert(0, ROOT)
    import bench
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [x for x in r.stdout.splitlines() if x.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["particles"] == 1048576


def test_reference_arm_loads_no_product_library():
    """The reference arm takes its SimParams from the reference's own loader
    (the recorded fixture) and runs the oracle: the product library is never
    mapped into the process."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '0']; sys.path.insert(0, %r); import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('PRODUCT_LOADED' if 'libpibiti_sph' in maps else 'PRODUCT_NOT_LOADED')") % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "PRODUCT_NOT_LOADED" in r.stdout


def test_reference_params_match_the_product_loader():
    """The recorded SimParams of the bench workload (the reference's loader)
    are the bytes the product's loader derives from the same element (the
    reference leaves SimParams::ff2 and the tail padding, the last 12 bytes,
    uninitialised)."""
    sys.path.insert(0, ROOT)
    import bench
    from pibiti_gb300 import configs
    from pibiti_gb300.sph import Scene
    xml = configs.dambreak_double().xml
    assert bench.reference_params(xml)[:548] == Scene.parse(xml).params.to_bytes()[:548]
