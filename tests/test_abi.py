"""The C-ABI library loads here (no GPU needed) and exports every function
include/*.h declares; the parameter struct has the reference's layout.
No compute call is made without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

from pibiti_gb300 import _lib
from pibiti_gb300.params import SimParams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(sph_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_library_loads():
    L = _lib.lib()
    assert L.sph_version().decode().startswith("pibiti_gb300")


def test_every_declared_function_is_exported():
    names = declared_functions("pibiti_sph.h")
    assert len(names) >= 30
    exported = exported_symbols(_lib.LIB_PATH)
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    # and the ctypes table covers them all
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_params_layout():
    assert ctypes.sizeof(SimParams) == 560
    assert SimParams.collPos.offset == 208 and SimParams.acc.offset == 292


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "pibiti_sph.h"\nint main(void){SimParams p; (void)p;'
                   ' return (int)sizeof(SimParams) - 560;}\n')
    exe = tmp_path / "t"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    assert subprocess.run([str(exe)]).returncode == 0


def test_errors_are_status_codes():
    """Argument errors come back as codes with a message, never an exit."""
    L = _lib.lib()
    assert L.sph_create(None, None) == 2
    assert "bad arguments" in _lib.last_error()
    assert L.sph_setParameters(None) == 2


def test_invalid_params_rejected():
    from pibiti_gb300.sph import Scene
    p = Scene.default().params
    p.rotType = 7
    with pytest.raises(_lib.SphError) as e:
        _lib.check(_lib.lib().sph_setParameters(ctypes.byref(p)))
    assert e.value.code == 3
    p = Scene.default().params
    p.numCells += 1
    with pytest.raises(_lib.SphError) as e:
        _lib.check(_lib.lib().sph_setParameters(ctypes.byref(p)))
    assert e.value.code == 3


def test_walk_shape_tables_match_header():
    """The Python tables of walk shapes cover exactly SPH_WALK_SHAPES shapes."""
    import os
    import re
    from pibiti_gb300.sph import SPH
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "pibiti_sph.h")).read()
    n = int(re.search(r"#define SPH_WALK_SHAPES (\d+)", hdr).group(1))
    assert len(SPH.WALK_THREADS) == len(SPH.WALK_STAGED) == len(SPH.WALK_KERNELS) == n
