"""The C ABI: the library builds for sm_103a, loads, exports every symbol include/dmsim.h declares,
and the ctypes mirror of every struct has the C layout.  No kernel is launched."""
import ctypes as C
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "dmsim.h"


def _declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dmsim_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from dmipy_sim_gb300 import _lib
    from dmipy_sim_gb300.build import build
    build()
    lib = C.CDLL(str(_lib.LIB_PATH))
    declared = _declared_functions()
    assert declared, "no functions found in include/dmsim.h"
    missing = [f for f in declared if not hasattr(lib, f)]
    assert not missing, f"declared but not exported: {missing}"
    assert set(_lib.EXPORTED) <= set(declared)
    lib.dmsim_version.restype = C.c_int
    assert lib.dmsim_version() == _lib.DMSIM_ABI_VERSION


def _c_layout(struct, fields):
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){",
           f'printf("%zu\\n", sizeof({struct}));']
    src += [f'printf("%zu\\n", offsetof({struct}, {f}));' for f in fields]
    src += ["return 0;}"]
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "l.c"
        c.write_text("\n".join(src))
        exe = Path(d) / "l"
        subprocess.run(["gcc", "-o", str(exe), str(c)], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    return [int(x) for x in out]


@pytest.mark.parametrize("cname,pyname", [("dmsim_geometry", "Geometry"),
                                          ("dmsim_walk_params", "WalkParams"),
                                          ("dmsim_walk_outputs", "WalkOutputs"),
                                          ("dmsim_batch_tuning", "BatchTuning"),
                                          ("dmsim_bloch_params", "BlochParams"),
                                          ("dmsim_mt_params", "MtParams"),
                                          ("dmsim_replay_bloch_params", "ReplayBlochParams"),
                                          ("dmsim_gemm", "Gemm"),
                                          ("dmsim_mlp_fwd", "MlpFwd")])
def test_struct_layout_matches_header(cname, pyname):
    from dmipy_sim_gb300 import _lib
    py = getattr(_lib, pyname)
    fields = [f[0] for f in py._fields_]
    got = _c_layout(cname, fields)
    assert got[0] == C.sizeof(py), f"sizeof({cname})"
    for f, off in zip(fields, got[1:]):
        assert getattr(py, f).offset == off, f"offset of {cname}.{f}"
