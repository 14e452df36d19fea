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


def test_tile_shapes_and_default_map():
    """The compiled tile shapes and the built-in map (host-only calls)."""
    lib = _lib.load()
    G = (ctypes.c_int32 * 64)()
    C = (ctypes.c_int32 * 64)()
    n = lib.bsb_tile_shapes(G, C, 64)
    assert n == _lib.BSB_NUM_TILES
    shapes = [(G[t], C[t]) for t in range(n)]
    assert len(set(shapes)) == n
    assert all(g in (4, 8, 16, 32) and c >= 1 for g, c in shapes)
    m = (ctypes.c_uint8 * _lib.BSB_TILE_MAP_LEN)()
    assert lib.bsb_get_tile_map(None, m, _lib.BSB_TILE_MAP_LEN) == 0
    for need in range(1, _lib.BSB_TILE_MAP_LEN):
        g, c = shapes[m[need]]
        assert g * c >= need, (need, g, c)
    # the widest query (1023 bases = 1024 columns) fits the widest shape
    assert max(g * c for g, c in shapes) == _lib.BSB_TILE_MAP_LEN - 1
    assert lib.bsb_get_tile_map(None, m, 10) == _lib.BSB_EINVAL
