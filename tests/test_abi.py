"""The C-ABI library builds, loads and exports every symbol include/*.h
declares; without a GPU it refuses to create a context (no CPU fallback)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from cabanamd_gb300 import gbmd
from cabanamd_gb300.build import build_lib

ROOT = Path(__file__).resolve().parents[1]


def _declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(gbmd_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib_path():
    return build_lib()


def test_every_declared_symbol_is_exported(lib_path):
    declared = _declared_functions()
    assert len(declared) >= 30
    lib = C.CDLL(str(lib_path))
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding wraps exactly the declared set
    assert set(gbmd.EXPORTS) == declared


def test_exports_are_c_linkage(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for n in _declared_functions():
        assert n in exported, n


def test_no_device_is_an_error_not_a_fallback(lib_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = gbmd.load_library()
    h = C.c_void_p()
    rc = lib.gbmd_create(C.byref(h), 0)
    assert rc == 7  # GBMD_ERR_NODEVICE
    assert not h.value
    with pytest.raises(gbmd.GbmdError):
        gbmd.Context(0)


def test_null_context_is_rejected(lib_path):
    lib = gbmd.load_library()
    assert lib.gbmd_set_units(None, 1.0, 1.0, 0.005) == 1
    assert lib.gbmd_last_error(None) == b"null context"
    assert lib.gbmd_version() >= 1
