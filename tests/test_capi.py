"""CPU checks of the C-ABI boundary: the library loads, exports every symbol that
include/cato_gpu.h declares, agrees with the oracle on configuration rules, and the ctypes
struct matches the C layout.  No GPU compute is called."""
import ctypes
import os
import re
import subprocess

import pytest

from fvleg_2d_gb300 import _lib
from fvleg_2d_gb300.config import CatoConfig, SchemeConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "cato_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cato_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("cato_gpu_create", "cato_gpu_integrate", "cato_gpu_get_timestep", "cato_gpu_solve",
              "cato_gpu_upload_primitive", "cato_gpu_download", "cato_gpu_run"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    L = _lib.load(build_if_missing=True)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_struct_layout(tmp_path):
    """The ctypes mirror has the C struct's size and every field's offset (compiled with gcc)."""
    names = [f[0] for f in CatoConfig._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"cato_gpu.h\"\n"
                   "int main(void) {\n  printf(\"%zu\\n\", sizeof(cato_config));\n"
                   + "".join(f'  printf("%zu\\n", offsetof(cato_config, {n}));\n' for n in names)
                   + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(CatoConfig)
    for n, off in zip(names, out[1:]):
        assert getattr(CatoConfig, n).offset == off, n


def test_config_defaults_match_deck_defaults(oracle):
    L = _lib.load(build_if_missing=True)
    c = CatoConfig()
    assert L.cato_config_default(ctypes.byref(c), 16, 8) == 0
    o = CatoConfig()
    assert oracle.lib().oracle_config_default(ctypes.byref(o), 16, 8) == 0
    assert bytes(c) == bytes(o)
    assert abs(c.gamma - 5.0 / 3.0) == 0 and c.cfl == 0.1 and c.apply_low_mach_fix == 1


@pytest.mark.parametrize("mutate,ok", [
    (lambda c: None, True),
    (lambda c: setattr(c, "n_ghost", 3), False),                  # TVD2 needs 2 ghost layers
    (lambda c: (setattr(c, "limiter", 4), setattr(c, "n_ghost", 3)), True),   # MLP5 needs 3
    (lambda c: setattr(c, "flux", 9), False),
    (lambda c: c.bc.__setitem__(0, 1), False),                    # +x symmetry, -x periodic
    (lambda c: setattr(c, "gamma", 1.0), False),
    (lambda c: setattr(c, "ni", 1), False),
])
def test_config_check_agrees_with_oracle(oracle, mutate, ok):
    L = _lib.load(build_if_missing=True)
    c = SchemeConfig(ni=16, nj=8, dx=0.1, dy=0.1).to_c()
    mutate(c)
    rc_lib = L.cato_config_check(ctypes.byref(c))
    rc_or = oracle.lib().oracle_config_check(ctypes.byref(c))
    assert rc_lib == rc_or
    assert (rc_lib == 0) == ok


def test_unknown_scheme_names_rejected():
    with pytest.raises(ValueError):
        SchemeConfig(ni=8, nj=8, dx=1, dy=1, flux_solver="FVLEG").to_c()
    with pytest.raises(ValueError):
        SchemeConfig(ni=8, nj=8, dx=1, dy=1, limiter="TVD5").to_c()
