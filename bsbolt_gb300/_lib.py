"""ctypes binding of libbsbgpu.so (the C ABI declared in include/bsbgpu.h).

The library is the product path: there is no CPU fallback.  If it is missing
or cannot be loaded, every call raises ``BsbError`` -- nothing silently
computes on the host.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbsbgpu.so")

BSB_OK = 0
BSB_EINVAL = -1
BSB_ECUDA = -2
BSB_ENOMEM = -3
BSB_EIO = -4
BSB_ETIMEOUT = -5
BSB_ETOOLONG = -6
BSB_ENOINDEX = -7
BSB_ECAPACITY = -8
BSB_NOALLOC_MAX_JOBS = 1 << 18
BSB_NUM_TILES = 61
BSB_ALIGN_STAGES = 6
BSB_TILE_MAP_LEN = 1025

# every extern "C" symbol include/bsbgpu.h declares
EXPORTS = (
    "bsb_ctx_create", "bsb_ctx_destroy", "bsb_last_error", "bsb_strerror", "bsb_ctx_stream",
    "bsb_extend_batch", "bsb_extend_batch_device", "bsb_sync", "bsb_last_kernel_ms",
    "bsb_probe_int_peak", "bsb_probe_int16x2_peak",
    "bsb_index_upload", "bsb_index_load", "bsb_seed_batch", "bsb_seed_batch_device",
    "bsb_sa_batch", "bsb_sa_batch_device", "bsb_extend_batch_noalloc", "bsb_align_regs_batch",
    "bsb_mem_align1_batch",
    "bsb_cost_features", "bsb_mlp_forward", "bsb_mlp_backward", "bsb_mlp_adam",
    "bsb_tile_shapes", "bsb_set_tile_map", "bsb_get_tile_map", "bsb_last_tile_ms", "bsb_index_full_sa",
    "bsb_index_upload_opac", "bsb_gen_cigar_batch", "bsb_align2_batch",
    "bsb_last_seed_extensions", "bsb_read_cost_log", "bsb_last_read_costs", "bsb_set_read_cost_model",
    "bsb_build_suffix_array", "bsb_last_stage_ms", "bsb_set_read_order_keys", "bsb_build_bwt",
)


class BsbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"bsbgpu error {code}: {msg}")
        self.code = code


class ExtParam(ctypes.Structure):
    """bsb_ext_param_t"""
    _fields_ = [("mat", ctypes.c_int8 * 25), ("pad_", ctypes.c_int8 * 3),
                ("o_del", ctypes.c_int32), ("e_del", ctypes.c_int32),
                ("o_ins", ctypes.c_int32), ("e_ins", ctypes.c_int32),
                ("zdrop", ctypes.c_int32)]


class SeedOpt(ctypes.Structure):
    """bsb_seed_opt_t"""
    _fields_ = [("min_seed_len", ctypes.c_int32), ("split_factor", ctypes.c_float),
                ("split_width", ctypes.c_int32), ("max_mem_intv", ctypes.c_int32)]


class IndexView(ctypes.Structure):
    """bsb_index_view_t"""
    _fields_ = [("primary", ctypes.c_uint64), ("L2", ctypes.c_uint64 * 5),
                ("bwt", ctypes.c_void_p), ("bwt_size", ctypes.c_uint64),
                ("sa", ctypes.c_void_p), ("n_sa", ctypes.c_uint64),
                ("sa_intv", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("pac", ctypes.c_void_p), ("l_pac", ctypes.c_int64),
                ("n_seqs", ctypes.c_int32), ("pad2_", ctypes.c_int32),
                ("ann_offset", ctypes.c_void_p), ("ann_len", ctypes.c_void_p)]


class AlignOpt(ctypes.Structure):
    """bsb_align_opt_t (mem_opt_t fields; BWA defaults as in mem_opt_init, bwamem.c:50-88)"""
    _fields_ = [(f, ctypes.c_int32) for f in ("a", "b", "o_del", "e_del", "o_ins", "e_ins", "w", "zdrop",
                                               "pen_clip5", "pen_clip3", "min_seed_len", "max_occ",
                                               "max_chain_gap", "min_chain_weight", "max_chain_extend")] + \
               [("mask_level", ctypes.c_float), ("drop_ratio", ctypes.c_float), ("split_factor", ctypes.c_float),
                ("split_width", ctypes.c_int32), ("max_mem_intv", ctypes.c_int32),
                ("mat", ctypes.c_int8 * 25), ("pad_", ctypes.c_int8 * 3), ("mask_level_redun", ctypes.c_float)]

    @classmethod
    def bwa_defaults(cls, a=1, b=4, o_del=6, e_del=1, o_ins=6, e_ins=1, w=100, zdrop=100, pen_clip5=5,
                     pen_clip3=5, min_seed_len=19, max_occ=500, split_width=10, max_mem_intv=20,
                     max_chain_gap=10000):
        o = cls(a=a, b=b, o_del=o_del, e_del=e_del, o_ins=o_ins, e_ins=e_ins, w=w, zdrop=zdrop,
                pen_clip5=pen_clip5, pen_clip3=pen_clip3, min_seed_len=min_seed_len, max_occ=max_occ,
                max_chain_gap=max_chain_gap, min_chain_weight=0, max_chain_extend=1 << 30, mask_level=0.5,
                drop_ratio=0.5, split_factor=1.5, split_width=split_width, max_mem_intv=max_mem_intv,
                mask_level_redun=0.95)
        for i in range(5):
            for j in range(5):
                o.mat[i * 5 + j] = -1 if (i == 4 or j == 4) else (a if i == j else -b)
        return o


_lib = None


def load(path: str = LIB_PATH):
    """Load libbsbgpu.so and declare its signatures (raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise BsbError(BSB_ECUDA, f"{path} is missing: run __graft_entry__.build() first "
                                  "(the CUDA library is required; there is no CPU fallback)")
    L = ctypes.CDLL(path)
    P, I64, I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    L.bsb_ctx_create.argtypes = [I32, ctypes.POINTER(P)]
    L.bsb_ctx_create.restype = I32
    L.bsb_ctx_destroy.argtypes = [P]
    L.bsb_ctx_destroy.restype = None
    L.bsb_last_error.argtypes = [P]
    L.bsb_last_error.restype = ctypes.c_char_p
    L.bsb_strerror.argtypes = [I32]
    L.bsb_strerror.restype = ctypes.c_char_p
    L.bsb_ctx_stream.argtypes = [P]
    L.bsb_ctx_stream.restype = P
    L.bsb_extend_batch.argtypes = [P, P, P, I64, P, I64, P, P]
    L.bsb_extend_batch.restype = I32
    L.bsb_extend_batch_device.argtypes = [P, P, P, I64, P, I64, P, P, P]
    L.bsb_extend_batch_device.restype = I32
    L.bsb_sync.argtypes = [P]
    L.bsb_sync.restype = I32
    L.bsb_probe_int_peak.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.bsb_probe_int_peak.restype = I32
    L.bsb_probe_int16x2_peak.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.bsb_probe_int16x2_peak.restype = I32
    L.bsb_index_upload.argtypes = [P, P]
    L.bsb_index_upload.restype = I32
    L.bsb_index_load.argtypes = [P, ctypes.c_char_p]
    L.bsb_index_load.restype = I32
    L.bsb_seed_batch.argtypes = [P, P, ctypes.c_int32, P, P, P, I64, P]
    L.bsb_seed_batch.restype = I32
    L.bsb_seed_batch_device.argtypes = [P, P, ctypes.c_int32, P, P, I64, ctypes.c_int32, P, P]
    L.bsb_seed_batch_device.restype = I32
    L.bsb_sa_batch.argtypes = [P, P, I64, P]
    L.bsb_sa_batch.restype = I32
    L.bsb_sa_batch_device.argtypes = [P, P, I64, P]
    L.bsb_sa_batch_device.restype = I32
    L.bsb_extend_batch_noalloc.argtypes = [P, P, I64, P, I64, P, P, P]
    L.bsb_extend_batch_noalloc.restype = I32
    L.bsb_align_regs_batch.argtypes = [P, P, ctypes.c_int32, P, P, P, I64, P]
    L.bsb_align_regs_batch.restype = I32
    L.bsb_mem_align1_batch.argtypes = [P, P, ctypes.c_int32, P, P, P, I64, P]
    L.bsb_mem_align1_batch.restype = I32
    L.bsb_cost_features.argtypes = [P, P, I64, P, I64, P]
    L.bsb_cost_features.restype = I32
    L.bsb_mlp_forward.argtypes = [P, P, P, I64, P, P]
    L.bsb_mlp_forward.restype = I32
    L.bsb_mlp_backward.argtypes = [P, P, P, P, ctypes.c_int32, P]
    L.bsb_mlp_backward.restype = I32
    L.bsb_mlp_adam.argtypes = [P, P, P, P, P, P, ctypes.c_float, ctypes.c_int32]
    L.bsb_mlp_adam.restype = I32
    L.bsb_last_kernel_ms.argtypes = [P]
    L.bsb_last_kernel_ms.restype = ctypes.c_float
    L.bsb_tile_shapes.argtypes = [P, P, I32]
    L.bsb_tile_shapes.restype = I32
    L.bsb_set_tile_map.argtypes = [P, P, I32]
    L.bsb_set_tile_map.restype = I32
    L.bsb_get_tile_map.argtypes = [P, P, I32]
    L.bsb_get_tile_map.restype = I32
    L.bsb_last_tile_ms.argtypes = [P, P, I32]
    L.bsb_last_tile_ms.restype = I32
    L.bsb_index_full_sa.argtypes = [P, I32]
    L.bsb_index_full_sa.restype = I32
    L.bsb_index_upload_opac.argtypes = [P, P, I64]
    L.bsb_index_upload_opac.restype = I32
    L.bsb_gen_cigar_batch.argtypes = [P, P, I64, I32, P, P, I64, P, I64, P, P, I64, ctypes.POINTER(I64)]
    L.bsb_gen_cigar_batch.restype = I32
    L.bsb_align2_batch.argtypes = [P, P, P, I64, P, I64, P]
    L.bsb_last_seed_extensions.argtypes = [P, ctypes.POINTER(I64)]
    L.bsb_last_seed_extensions.restype = I32
    L.bsb_set_read_order_keys.argtypes = [P, P, I32]
    L.bsb_set_read_order_keys.restype = I32
    L.bsb_last_stage_ms.argtypes = [P, P, I32]
    L.bsb_last_stage_ms.restype = I32
    L.bsb_read_cost_log.argtypes = [P, I32]
    L.bsb_read_cost_log.restype = I32
    L.bsb_last_read_costs.argtypes = [P, ctypes.c_int32, P, P]
    L.bsb_last_read_costs.restype = I32
    L.bsb_set_read_cost_model.argtypes = [P, P]
    L.bsb_set_read_cost_model.restype = I32
    L.bsb_build_suffix_array.argtypes = [P, P, I64, P]
    L.bsb_build_suffix_array.restype = I32
    L.bsb_build_bwt.argtypes = [P, P, I64, I32, I64, P, P, P]
    L.bsb_build_bwt.restype = I32
    L.bsb_align2_batch.restype = I32
    _lib = L
    return L


def check(ctx, rc: int):
    if rc != 0:
        L = load()
        msg = L.bsb_last_error(ctx).decode() if ctx else L.bsb_strerror(rc).decode()
        raise BsbError(rc, msg or L.bsb_strerror(rc).decode())
    return rc
