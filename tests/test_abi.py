"""CPU checks of the drop-in boundary: libtp.so builds, loads and exports every
entry point that include/tp.h declares (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "tp.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^tp_status\s+(tp_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("tp_create", "tp_destroy", "tp_set_tasks", "tp_set_kernels", "tp_set_image", "tp_convert_correct",
              "tp_imclt", "tp_get_rbg", "tp_correlate", "tp_extract"):
        assert s in syms


def test_library_exports_all_symbols():
    import build as tp_build
    lib = ctypes.CDLL(tp_build.build())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, "not exported: %s" % missing


def test_python_binding_covers_header():
    from tileproc import _lib
    assert set(declared_symbols()) <= set(_lib.PROTOTYPES), set(declared_symbols()) - set(_lib.PROTOTYPES)


def test_create_without_gpu_fails_cleanly():
    """With no CUDA device tp_create reports TP_ERR_NOT_BUILT instead of crashing."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    from tileproc import _lib
    L = _lib.load()
    cfg = _lib.TpConfig(4, 1, 64, 64, 0, 0, 16, 0, 1, 0)
    h = ctypes.c_void_p()
    st = L.tp_create(ctypes.byref(cfg), ctypes.byref(h))
    assert st != _lib.TP_OK and not h.value


def test_argument_validation_without_gpu():
    from tileproc import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.tp_create(None, ctypes.byref(h)) == _lib.TP_ERR_ARG
    bad = _lib.TpConfig(0, 1, 64, 64, 0, 0, 16, 0, 1, 0)
    assert L.tp_create(ctypes.byref(bad), ctypes.byref(h)) == _lib.TP_ERR_ARG
    bad = _lib.TpConfig(4, 2, 64, 64, 0, 0, 16, 0, 1, 0)
    assert L.tp_create(ctypes.byref(bad), ctypes.byref(h)) == _lib.TP_ERR_ARG
    bad = _lib.TpConfig(4, 1, 60, 64, 0, 0, 16, 0, 1, 0)
    assert L.tp_create(ctypes.byref(bad), ctypes.byref(h)) == _lib.TP_ERR_ARG
    p = _lib.TpCorrParams()
    assert L.tp_default_corr_params(ctypes.byref(p)) == _lib.TP_OK
    assert abs(p.fat_zero - 0.05) < 1e-7 and p.corr_strip_hight == 9
    pairs = (_lib.TpPair * 6)()
    n = ctypes.c_int()
    assert L.tp_quad_pairs(pairs, ctypes.byref(n)) == _lib.TP_OK and n.value == 6
    assert [(pairs[i].cam1, pairs[i].cam2, pairs[i].kind) for i in range(6)] == \
        [(0, 1, 0), (2, 3, 0), (0, 2, 1), (1, 3, 1), (0, 3, 2), (2, 1, 3)]


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror of an include/tp.h struct has the C layout: sizeof and each field's offset,
    from a probe compiled against the header with the host compiler."""
    import shutil
    import subprocess
    from tileproc import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [("tp_config", _lib.TpConfig), ("tp_geometry", _lib.TpGeometry), ("tp_rig_offset", _lib.TpRigOffset),
             ("tp_pair", _lib.TpPair), ("tp_corr_params", _lib.TpCorrParams),
             ("tp_texture_params", _lib.TpTextureParams), ("tp_lma_params", _lib.TpLmaParams)]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "tp.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (l.split() for l in out if l.strip())}
    for cname, py in pairs:
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
