"""ctypes binding of the C ABI in include/prodm_gb300.h.

The CUDA library is in-tree (prodm_gb300/libprodm_gb300.so, built by
prodm_gb300/build.py). There is no CPU fallback: if the library is missing or
fails to load, every entry point raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libprodm_gb300.so")

F32, F64 = 0, 1
ENC = {"negabinary": 0, "grouped": 1, "perbit": 2}
BASIS = {"hierarchical": 0, "orthogonal": 1}
INTERP = {"greedy": 0, "sign_exclude": 1, "negabinary": 2}
EST = {"max_hb": 0, "max_ob": 1, "l2_hb": 2, "snorm": 3}
COLLECT = {"max": 0, "squared": 1}
STATUS = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ETIMEOUT", 5: "ECORRUPT", 6: "EUNSUPPORTED"}


class ProdmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class prodm_config(C.Structure):
    _fields_ = [("dtype", C.c_int), ("ndims", C.c_int), ("dims", C.c_uint32 * 3), ("target_level", C.c_int),
                ("num_bitplanes", C.c_int), ("encoder", C.c_int), ("basis", C.c_int), ("collector", C.c_int)]


_P = C.c_void_p
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_u8p = C.POINTER(C.c_uint8)
_dp = C.POINTER(C.c_double)
_i = C.c_int

_SIGS = {
    "prodm_last_error_string": (C.c_char_p, []),
    "prodm_version": (_i, []),
    "prodm_max_level": (_i, [_i, _u32p, C.POINTER(_i)]),
    "prodm_level_dims": (_i, [_i, _u32p, _i, _u32p, _u64p]),
    "prodm_decompose_workspace": (_i, [_i, _i, _u32p, C.c_uint32, _i, C.POINTER(C.c_size_t)]),
    "prodm_decompose": (_i, [_i, _P, _i, _u32p, C.c_uint32, _u32p, _i, _P, C.c_size_t, _P]),
    "prodm_recompose": (_i, [_i, _P, _i, _u32p, C.c_uint32, _u32p, _i, _P, C.c_size_t, _P]),
    "prodm_interleave": (_i, [_i, _P, _i, _u32p, _u32p, _u32p, _P, _u32p, _P]),
    "prodm_reposition": (_i, [_i, _P, _i, _u32p, _u32p, _u32p, _P, _u32p, _P]),
    "prodm_encode_bound": (_i, [_i, _i, C.c_uint64, _i, _u64p]),
    "prodm_encode_workspace": (_i, [_i, _i, C.c_uint64, _i, C.POINTER(C.c_size_t)]),
    "prodm_encode": (_i, [_i, _i, _P, C.c_uint64, _i, _i, _P, C.c_uint64, _P, _P, _P, C.c_size_t, _P]),
    "prodm_decoder_create": (_i, [C.POINTER(_P), _i, _i]),
    "prodm_progressive_decode": (_i, [_P, _P, _u32p, C.c_uint64, _i, _i, _i, _i, _i, _P, _P]),
    "prodm_decoder_destroy": (_i, [_P]),
    "prodm_collect_max": (_i, [_i, C.c_double, _i, _dp]),
    "prodm_collect_squared_workspace": (_i, [_i, _i, C.POINTER(C.c_size_t)]),
    "prodm_collect_squared": (_i, [_i, _P, C.c_uint64, _i, C.c_double, _P, _P, C.c_size_t, _P]),
    "prodm_collect_squared_noalloc": (_i, [_i, _P, C.c_uint64, _i, C.c_double, _P, _P]),
    "prodm_recompose_packed_workspace": (_i, [_i, _i, _u32p, C.c_uint32, C.POINTER(C.c_size_t)]),
    "prodm_recompose_packed": (_i, [_i, _P, _i, _u32p, C.c_uint32, _P, _P, C.c_size_t, _P]),
    "prodm_recompose_adjoint": (_i, [_i, _P, _i, _u32p, C.c_uint32, _P, _P, C.c_size_t, _P]),
    "prodm_recompose_packed_basis_workspace": (_i, [_i, _i, _i, _u32p, C.c_uint32, C.POINTER(C.c_size_t)]),
    "prodm_recompose_packed_basis": (_i, [_i, _i, _P, _i, _u32p, C.c_uint32, _P, _P, C.c_size_t, _P]),
    "prodm_recompose_adjoint_basis": (_i, [_i, _i, _P, _i, _u32p, C.c_uint32, _P, _P, C.c_size_t, _P]),
    "prodm_qoi_ge_values": (_i, [_i, _P, _P, _P, _P, _P, C.c_uint64, _P, _P, _P, _P, _P, _P, _P]),
    "prodm_qoi_ge_bounds": (_i, [_i, _P, _P, _P, _P, _P, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, _P, _P, _P, _P]),
    "prodm_lossless_compress_bound": (_i, [_u32p, _i, _u64p]),
    "prodm_lossless_compress_level": (_i, [_P, _u32p, _i, _i, _P, C.c_uint64, _u32p, C.POINTER(_i), _P]),
    "prodm_lossless_decompress_level": (_i, [_P, _u32p, _i, _i, _i, _i, _P, C.c_uint64, _u32p, _P]),
    "prodm_interpret": (_i, [_i, _i, _i, _i, _i, C.c_double, _i, _i, _P, _P, C.c_double, _P, _P, _P]),
    "prodm_mdr_create": (_i, [C.POINTER(_P), C.POINTER(prodm_config)]),
    "prodm_mdr_refactor": (_i, [_P, _P, _P]),
    "prodm_mdr_level_info": (_i, [_P, _u32p, _dp, _dp, _P]),
    "prodm_mdr_metadata": (_i, [_P, _u8p, C.c_size_t, C.POINTER(C.c_size_t), _P]),
    "prodm_mdr_export_level": (_i, [_P, _i, _P, C.c_uint64, _i, _u64p, _P]),
    "prodm_mdr_set_lossless": (_i, [_P, _i, _P]),
    "prodm_mdr_set_zstd_latter": (_i, [_P, _i]),
    "prodm_mdr_export_level_range": (_i, [_P, _i, C.c_uint64, C.c_uint64, _P, _i, _P]),
    "prodm_mdr_load_level_file": (_i, [_P, _i, C.c_char_p, C.c_uint64, C.c_uint64, C.c_uint64, _P]),
    "prodm_mdr_write_level_file": (_i, [_P, _i, C.c_char_p, _P]),
    "prodm_mdr_file_read_mode": (_i, [_P, C.POINTER(_i)]),
    "prodm_mdr_retrieve": (_i, [_P, C.c_double, _i, _i, C.c_double, _P, _P]),
    "prodm_mdr_retrieve_planes": (_i, [_P, _u8p, _P, _P]),
    "prodm_mdr_interpret": (_i, [_P, C.c_double, _i, _i, C.c_double, _P]),
    "prodm_mdr_reconstruct": (_i, [_P, _P, _P]),
    "prodm_mdr_load_metadata": (_i, [_P, _u8p, C.c_size_t, _P]),
    "prodm_mdr_load_level": (_i, [_P, _i, _P, C.c_uint64, C.c_uint64, _i, _P]),
    "prodm_mdr_get_index": (_i, [_P, _u8p, _P]),
    "prodm_mdr_reset_retrieval": (_i, [_P, _P]),
    "prodm_mdr_status": (_i, [_P, _P]),
    "prodm_debug_tile_wait": (_i, [_i, C.c_longlong]),
    "prodm_mdr_coefficients": (_i, [_P, _P, _P]),
    "prodm_mdr_destroy": (_i, [_P]),
    "prodm_batch_create": (_i, [C.POINTER(_P), _i, C.POINTER(prodm_config)]),
    "prodm_batch_bind": (_i, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "prodm_batch_set_launch": (_i, [_P, _i, _i]),
    "prodm_batch_set_stage_launch": (_i, [_P, _i, _i, _i]),
    "prodm_batch_refactor": (_i, [_P, _P]),
    "prodm_batch_set_tolerances": (_i, [_P, _dp, _P]),
    "prodm_batch_retrieve": (_i, [_P, _i, _i, C.c_double, _P]),
    "prodm_batch_reset": (_i, [_P, _P]),
    "prodm_batch_status": (_i, [_P, _P]),
    "prodm_batch_set_fused_unit": (_i, [_P, _i]),
    "prodm_batch_field_info": (_i, [_P, _i, _u8p, _u32p, _dp, _P]),
    "prodm_batch_export_level": (_i, [_P, _i, _i, _P, C.c_uint64, _i, _u64p, _P]),
    "prodm_batch_destroy": (_i, [_P]),
    "prodm_mdr_set_timing": (_i, [_P, _i]),
    "prodm_mdr_stage_times": (_i, [_P, _dp, _u32p]),
    "prodm_kernel_launch_count": (_i, [_u64p]),
}

_lib = None


def load():
    """Load the library (raises if it is absent: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("prodm_gb300: %s is missing; run prodm_gb300/build.py (or __graft_entry__.build())"
                              % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def declared_symbols():
    return list(_SIGS)


def check(rc):
    if rc != 0:
        msg = load().prodm_last_error_string()
        raise ProdmError(rc, msg.decode() if msg else "")
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args))
