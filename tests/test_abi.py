"""The C-ABI library loads and exports every entry point the header declares."""
import ctypes
import os
import re

from gpuocean_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gpuocean_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(goc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "goc_cdklm_rk2_step" in names and "goc_max_dt" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_params_struct_matches_header_fields():
    text = open(HEADER).read()
    body = text[text.index("typedef struct GocCdklmParams"):text.index("} GocCdklmParams;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = re.findall(r"\*?\s*([a-z_0-9]+)\s*[,;]", body.split("{", 1)[1])
    assert [f[0] for f in _lib.GocCdklmParams._fields_] == names


def test_argument_validation_without_gpu():
    # validation happens before any CUDA call
    lib = _lib.load()
    p = _lib.GocCdklmParams()
    p.nx, p.ny = 0, 4
    rc = lib.goc_cdklm_rk2_step(ctypes.byref(p), 1.0, None, None, None, None, None, None, 64, None, 64, None, 64, None)
    assert rc == -1 and "nx, ny" in _lib.last_error()
    assert lib.goc_max_dt_partials(256, 256) == 8 * 32
    rc = lib.goc_max_dt(8, 8, 1.0, 1.0, 9.8, None, None, None, 48, None, 48, 1e20, None, 0, None, None)
    assert rc == -1
