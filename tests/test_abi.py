"""The C-ABI library loads without a GPU and exports every entry point that
include/hyperflow_gpu.h declares; the Python binding covers all of them."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "hyperflow_gpu.h")).read()
    return sorted(set(re.findall(r"^HF_EXPORT [^(]*?\b(hf_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from hyperflow_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared()
    for must in ("hf_init", "hf_fill_ghosts", "hf_flux_update", "hf_chem_advance", "hf_cfl_dt", "hf_validate",
                 "hf_interp_coarse_to_fine", "hf_properties", "hf_hllc", "hf_stepper_step"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from hyperflow_gb300 import _lib
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(declared()) <= bound, set(declared()) - bound


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of hf_level / hf_patch / hf_counters match the C compiler's layout."""
    import subprocess
    from hyperflow_gb300 import _lib
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "hyperflow_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(hf_level), offsetof(hf_level, inlet), offsetof(hf_level, wedge_start),
         sizeof(hf_patch), offsetof(hf_patch, offset), sizeof(hf_counters));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(_lib.Level), _lib.Level.inlet.offset, _lib.Level.wedge_start.offset,
            ctypes.sizeof(_lib.Patch), _lib.Patch.offset.offset, ctypes.sizeof(_lib.Counters)]
    assert got == want


def test_init_rejects_unknown_mechanism(lib):
    lib.hf_init.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    h = ctypes.c_void_p()
    assert lib.hf_init(b"gri30.yaml", 0, ctypes.byref(h)) == 4  # HF_ERR_ARG, before touching a device
    assert not h.value


def test_every_struct_mirror_matches_header(tmp_path):
    """Every ctypes mirror of a header struct: sizeof and the offset of every named field
    as the C compiler lays them out."""
    import subprocess
    from hyperflow_gb300 import _lib
    mirrors = {"hf_level": _lib.Level, "hf_patch": _lib.Patch, "hf_counters": _lib.Counters,
               "hf_chem_history": _lib.ChemHistory, "hf_adjoint_opts": _lib.AdjointOpts,
               "hf_tag_criteria": _lib.TagCriteria, "hf_amr_opts": _lib.AmrOpts}
    lines, want = [], []
    for cname, py in mirrors.items():
        lines.append('  printf("%%zu\\n", sizeof(%s));' % cname)
        want.append(ctypes.sizeof(py))
        for f in py._fields_:
            if f[0].startswith("pad"):
                continue
            lines.append('  printf("%%zu\\n", offsetof(%s, %s));' % (cname, f[0]))
            want.append(getattr(py, f[0]).offset)
    src = tmp_path / "layouts.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"hyperflow_gpu.h\"\nint main(void) {\n" +
                   "\n".join(lines) + "\n  return 0;\n}\n")
    exe = tmp_path / "layouts"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want


def test_every_entry_point_rejects_null_arguments(lib):
    """With null handles and pointers and zero sizes every status-returning entry point
    returns HF_ERR_ARG before touching a device, and the others do nothing (no GPU is
    needed for this)."""
    from hyperflow_gb300 import _lib
    for name, res, args in _lib.SIGNATURES:
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
        vals = [0.0 if a is ctypes.c_double else 0 if a in (ctypes.c_int, ctypes.c_int32, ctypes.c_int64) else None
                for a in args]
        r = f(*vals)
        if name == "hf_nspecies":
            assert r == 0
        elif name == "hf_set_chem_tuning":
            assert r == 0  # zeros leave both settings as they are; it takes no handle or pointer
        elif res is _lib.SIGNATURES[0][1]:
            assert r == _lib.HF_ERR_ARG, name
