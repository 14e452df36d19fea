"""The C ABI library loads and exports every symbol include/*.h declares (CPU only;
no compute call is made without a GPU)."""
import ctypes
import glob
import os
import re

from bsbolt_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(bsb_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return syms


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert {"bsb_ctx_create", "bsb_extend_batch", "bsb_extend_batch_device"} <= syms


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, f"not exported: {missing}"
    assert set(_lib.EXPORTS) <= declared_symbols()


def test_error_strings_and_no_device_behaviour():
    lib = _lib.load()
    assert lib.bsb_strerror(-1) == b"invalid argument"
    assert lib.bsb_strerror(-6) == b"sequence too long"
    # NULL out-pointer is rejected before any CUDA call
    assert lib.bsb_ctx_create(0, None) == _lib.BSB_EINVAL
    assert lib.bsb_last_error(None) == b"no context"
