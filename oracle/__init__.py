"""CPU oracle for the MDR path -- test infrastructure only.

Python bindings (ctypes + numpy) for the oracle restatement
(``libmdr_oracle.so``) and, where it was built, for the reference harness
(``_ref/libprodm_ref.so``). Only tests, the smoke check and the benchmark's
CPU-baseline leg import this package; the product library never does.
"""
import ctypes as C
import os

import numpy as np

from .build_oracle import ORACLE_SO, REF_SO, build_oracle, build_ref

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")

ENCODERS = {"negabinary": 0, "grouped": 1, "perbit": 2}
INTERPRETERS = {"greedy": 0, "sign_exclude": 1, "negabinary": 2}
ESTIMATORS = {"max_hb": 0, "max_ob": 1, "l2_hb": 2, "snorm": 3}


def _sfx(dtype):
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def _tp(dtype):
    return _f32p if np.dtype(dtype) == np.float32 else _f64p


def _ct(dtype):
    return C.c_float if np.dtype(dtype) == np.float32 else C.c_double


def stream_capacity(n, B, dtype):
    """Upper bound on the bytes one level's streams can take."""
    bs = 32 if np.dtype(dtype) == np.float32 else 64
    nb = (n + bs - 1) // bs
    return B * (2 * nb + 2) * (bs // 8) + 4 + nb + 64


class _Lib:
    prefix = "or"

    def __init__(self, path):
        self.lib = C.CDLL(path)
        self._setup()

    def _fn(self, name, restype, *args):
        f = getattr(self.lib, name)
        f.restype = restype
        f.argtypes = list(args)
        return f

    def _setup(self):
        pass


class Oracle(_Lib):
    """The oracle restatement (oracle/mdr_oracle.hpp)."""

    def _setup(self):
        L = self.lib
        L.or_max_level.restype = C.c_int
        L.or_max_level.argtypes = [C.c_int, _u32p]
        L.or_level_dims.argtypes = [C.c_int, _u32p, C.c_int, _u32p]
        L.or_level_elements.argtypes = [C.c_int, _u32p, C.c_int, _u32p]

    # geometry -----------------------------------------------------------
    def max_level(self, dims):
        d = np.asarray(dims, np.uint32)
        return self.lib.or_max_level(len(d), d)

    def level_dims(self, dims, L):
        d = np.asarray(dims, np.uint32)
        out = np.zeros((L + 1) * len(d), np.uint32)
        self.lib.or_level_dims(len(d), d, L, out)
        return out.reshape(L + 1, len(d))

    def level_elements(self, dims, L):
        d = np.asarray(dims, np.uint32)
        out = np.zeros(L + 1, np.uint32)
        self.lib.or_level_elements(len(d), d, L, out)
        return out

    # interleaver --------------------------------------------------------
    def interleave(self, data, dims, fine, coarse):
        s = _sfx(data.dtype)
        f = self._fn("or_interleave_" + s, None, _tp(data.dtype), C.c_int, _u32p, _u32p, _u32p, _tp(data.dtype))
        fine = np.asarray(fine, np.uint32); coarse = np.asarray(coarse, np.uint32)
        n = int(np.prod(fine.astype(np.int64))) - int(np.prod(coarse.astype(np.int64)))
        buf = np.zeros(n, data.dtype)
        f(np.ascontiguousarray(data), len(dims), np.asarray(dims, np.uint32), fine, coarse, buf)
        return buf

    def reposition(self, buf, data, dims, fine, coarse):
        s = _sfx(buf.dtype)
        f = self._fn("or_reposition_" + s, None, _tp(buf.dtype), C.c_int, _u32p, _u32p, _u32p, _tp(buf.dtype))
        f(np.ascontiguousarray(buf), len(dims), np.asarray(dims, np.uint32), np.asarray(fine, np.uint32),
          np.asarray(coarse, np.uint32), data)
        return data

    # encoders -------------------------------------------------------------
    def encode(self, kind, data, exp, B, collect=False):
        """Returns (blob bytes as uint8 array, sizes[B], errors[B+1] or None)."""
        s = _sfx(data.dtype)
        name = ("%s_nb_encode_" if kind == "negabinary" else "%s_gr_encode_") % self.prefix + s
        f = self._fn(name, C.c_int64, _tp(data.dtype), C.c_uint64, C.c_int, C.c_int, _u8p, _u32p, C.c_void_p)
        blob = np.zeros(stream_capacity(len(data), B, data.dtype), np.uint8)
        sizes = np.zeros(B, np.uint32)
        errs = np.zeros(B + 1, np.float64) if collect else None
        total = f(np.ascontiguousarray(data), len(data), int(exp), int(B), blob, sizes,
                  errs.ctypes.data if collect else None)
        return blob[:total].copy(), sizes, errs

    def pb_encode(self, data, exp, B):
        """PerBit streams of one level: (blob bytes, sizes[B])."""
        f = self._fn("%s_pb_encode_%s" % (self.prefix, _sfx(data.dtype)), C.c_int64, _tp(data.dtype), C.c_uint64,
                     C.c_int, C.c_int, _u8p, _u32p)
        n = len(data)
        blob = np.zeros(B * (2 * n // 8 + 8) + 64, np.uint8)
        sizes = np.zeros(B, np.uint32)
        total = f(np.ascontiguousarray(data), n, int(exp), int(B), blob, sizes)
        return blob[:total].copy(), sizes

    # lossless stage ------------------------------------------------------
    def adaptive_stopping(self, raw_sizes, comp_sizes, latter=26):
        """(stopping index, compressed flags) of AdaptiveLevelCompressor's rule."""
        raw = np.ascontiguousarray(raw_sizes, np.uint32)
        comp = np.ascontiguousarray(comp_sizes, np.uint32)
        flags = np.zeros(len(raw), np.uint8)
        f = self._fn("or_adaptive_stopping", C.c_int, _u32p, _u32p, C.c_int, C.c_int, _u8p)
        return f(raw, comp, len(raw), int(latter), flags), flags

    def zcb_compress(self, raw):
        raw = np.ascontiguousarray(raw, np.uint8)
        size = self._fn("or_zcb_size", C.c_uint64, _u8p, C.c_uint64)(raw, raw.size)
        out = np.zeros(max(int(size), 1), np.uint8)
        n = self._fn("or_zcb_compress", C.c_uint64, _u8p, C.c_uint64, _u8p)(raw, raw.size, out)
        assert n == size
        return out[:n]

    def zcb_decompress(self, comp, cap):
        comp = np.ascontiguousarray(comp, np.uint8)
        out = np.zeros(max(int(cap), 1), np.uint8)
        n = self._fn("or_zcb_decompress", C.c_int64, _u8p, C.c_uint64, _u8p, C.c_uint64)(comp, comp.size, out, cap)
        if n < 0:
            raise ValueError("malformed ZCB stream")
        return out[:n]

    def perbit_state(self, dtype):
        """Stateful PerBit progressive decoder (one per encoder object)."""
        return _PerBitState(self, dtype)

    def nb_decode(self, blob, sizes, n, exp, s, num, dtype):
        f = self._fn("or_nb_decode_" + _sfx(dtype), C.c_int, _u8p, _u32p, C.c_uint64, C.c_int, C.c_int, C.c_int,
                     _tp(dtype))
        out = np.zeros(n, dtype)
        f(np.ascontiguousarray(blob, np.uint8), np.ascontiguousarray(sizes, np.uint32), n, exp, s, num, out)
        return out

    def grouped_state(self, dtype):
        return _GroupedState(self, dtype)

    def max_collect(self, bound, B, dtype):
        f = self._fn("or_max_collect_" + _sfx(dtype), None, _ct(dtype), C.c_int, _f64p)
        out = np.zeros(B + 1, np.float64)
        f(bound, B, out)
        return out

    def sq_collect(self, data, B, maxv):
        f = self._fn("or_sq_collect_" + _sfx(data.dtype), None, _tp(data.dtype), C.c_uint64, C.c_int, _ct(data.dtype),
                     _f64p)
        out = np.zeros(B + 1, np.float64)
        f(np.ascontiguousarray(data), len(data), B, maxv, out)
        return out

    def max_abs(self, data):
        f = self._fn("or_max_abs_" + _sfx(data.dtype), _ct(data.dtype), _tp(data.dtype), C.c_uint64)
        return f(np.ascontiguousarray(data), len(data))

    def interpret(self, kind, est, sizes, errs, tol, index, ndims=3, L=None, s=0.0, dtype=np.float32):
        sizes = np.ascontiguousarray(sizes, np.uint32)
        errs = np.ascontiguousarray(errs, np.float64)
        nl, B = sizes.shape
        if L is None:
            L = nl - 1
        f = self._fn("%s_interpret_%s" % (self.prefix, _sfx(dtype)), None, C.c_int, C.c_int, C.c_int, C.c_int,
                     C.c_double, C.c_int, C.c_int, _u32p, _f64p, C.c_double, _u8p, _u32p)
        idx = np.ascontiguousarray(index, np.uint8).copy()
        rsz = np.zeros(nl, np.uint32)
        f(INTERPRETERS[kind], ESTIMATORS[est], ndims, L, s, nl, B, sizes, errs, tol, idx, rsz)
        return idx, rsz

    # MGARD ----------------------------------------------------------------
    def decompose(self, data, dims, L, hierarchical=True):
        f = self._fn("or_decompose_" + _sfx(data.dtype), None, _tp(data.dtype), C.c_int, _u32p, C.c_int, C.c_int)
        out = np.ascontiguousarray(data).copy()
        f(out, len(dims), np.asarray(dims, np.uint32), L, int(hierarchical))
        return out

    def recompose(self, data, dims, L, hierarchical=True):
        f = self._fn("or_recompose_" + _sfx(data.dtype), None, _tp(data.dtype), C.c_int, _u32p, C.c_int, C.c_int)
        out = np.ascontiguousarray(data).copy()
        f(out, len(dims), np.asarray(dims, np.uint32), L, int(hierarchical))
        return out

    def recompose_packed(self, packed, dims, L, hierarchical=True):
        """packed level coefficients -> natural field (the forward of the adjoint pair)."""
        t = packed.dtype
        f = self._fn("or_recompose_packed_" + _sfx(t), None, _tp(t), C.c_int, _u32p, C.c_int, C.c_int, _tp(t))
        out = np.zeros(int(np.prod(dims)), t)
        f(np.ascontiguousarray(packed), len(dims), np.asarray(dims, np.uint32), L, int(hierarchical), out)
        return out.reshape(tuple(dims))

    def recompose_adjoint(self, grad, dims, L):
        """transpose of recompose_packed (hierarchical basis)."""
        t = grad.dtype
        f = self._fn("or_recompose_adjoint_" + _sfx(t), None, _tp(t), C.c_int, _u32p, C.c_int, _tp(t))
        out = np.zeros(int(np.prod(dims)), t)
        f(np.ascontiguousarray(grad).ravel(), len(dims), np.asarray(dims, np.uint32), L, out)
        return out

    # GE quantities of interest (double) ----------------------------------
    def qoi_values(self, vx, vy, vz, p, d):
        """V_TOT, T, C, Mach, PT, mu (six arrays)."""
        pre = self.prefix
        a = [np.ascontiguousarray(x, np.float64) for x in (vx, vy, vz, p, d)]
        n = a[0].size
        outs = [np.zeros(n) for _ in range(6)]
        dp = C.POINTER(C.c_double)
        f = self._fn(pre + "_qoi_values_f64", None, *([_tp(np.float64)] * 5), C.c_uint64, *([_tp(np.float64)] * 6))
        f(*a, n, *outs)
        return outs

    def qoi_vtot_bound(self, vx, vy, vz, ebs):
        pre = self.prefix
        a = [np.ascontiguousarray(x, np.float64) for x in (vx, vy, vz)]
        out = np.zeros(a[0].size)
        f = self._fn(pre + "_qoi_vtot_bound_f64", None, *([_tp(np.float64)] * 3), C.c_uint64, C.c_double,
                     C.c_double, C.c_double, _tp(np.float64))
        f(*a, a[0].size, float(ebs[0]), float(ebs[1]), float(ebs[2]), out)
        return out

    def qoi_t_bound(self, p, d, eb_p, eb_d):
        pre = self.prefix
        a = [np.ascontiguousarray(x, np.float64) for x in (p, d)]
        out = np.zeros(a[0].size)
        f = self._fn(pre + "_qoi_t_bound_f64", None, _tp(np.float64), _tp(np.float64), C.c_uint64, C.c_double,
                     C.c_double, _tp(np.float64))
        f(*a, a[0].size, float(eb_p), float(eb_d), out)
        return out

    # composed -------------------------------------------------------------
    def refactor(self, field, L, B, encoder="negabinary", hierarchical=True, collect=False):
        """Composed refactor. Returns dict(blob, sizes[L+1,B], bounds[L+1], errs, coeffs)."""
        dims = np.asarray(field.shape, np.uint32)
        dt = field.dtype
        le = self.level_elements(dims, L)
        cap = sum(stream_capacity(int(n), B, dt) for n in le)
        blob = np.zeros(cap, np.uint8)
        sizes = np.zeros((L + 1) * B, np.uint32)
        bounds = np.zeros(L + 1, dt)
        errs = np.zeros((L + 1) * (B + 1), np.float64)
        coeffs = np.zeros(field.size, dt)
        f = self._fn("or_refactor_" + _sfx(dt), C.c_int64, _tp(dt), C.c_int, _u32p, C.c_int, C.c_int, C.c_int,
                     C.c_int, C.c_int, _u8p, _u32p, _tp(dt), _f64p, _tp(dt))
        total = f(np.ascontiguousarray(field).ravel(), len(dims), dims, L, B, ENCODERS[encoder], int(hierarchical),
                  int(collect), blob, sizes, bounds, errs, coeffs)
        if total < 0:
            raise ValueError("oracle refactor rejected the request (%d)" % total)
        return dict(blob=blob[:total].copy(), sizes=sizes.reshape(L + 1, B), bounds=bounds,
                    errs=errs.reshape(L + 1, B + 1) if collect else None, coeffs=coeffs.reshape(field.shape))

    def retrieve(self, shape, L, B, blob, sizes, bounds, index, encoder="negabinary", hierarchical=True,
                 dtype=np.float32):
        dims = np.asarray(shape, np.uint32)
        out = np.zeros(int(np.prod(shape)), dtype)
        f = self._fn("or_retrieve_" + _sfx(dtype), C.c_int, C.c_int, _u32p, C.c_int, C.c_int, C.c_int, C.c_int,
                     _u8p, _u32p, _tp(dtype), _u8p, _tp(dtype))
        rc = f(len(dims), dims, L, B, ENCODERS[encoder], int(hierarchical), np.ascontiguousarray(blob, np.uint8),
               np.ascontiguousarray(sizes, np.uint32).ravel(), np.ascontiguousarray(bounds, dtype),
               np.ascontiguousarray(index, np.uint8), out)
        if rc != 0:
            raise ValueError("oracle retrieve failed (%d)" % rc)
        return out.reshape(shape)


class _GroupedState:
    def __init__(self, lib, dtype):
        self.lib, self.dtype, self.sfx = lib, np.dtype(dtype), _sfx(dtype)
        pre = lib.prefix
        new = lib._fn("%s_gr_state_new_%s" % (pre, self.sfx), C.c_void_p)
        self._free = lib._fn("%s_gr_state_free_%s" % (pre, self.sfx), None, C.c_void_p)
        self._dec = lib._fn("%s_gr_decode_%s" % (pre, self.sfx), C.c_int, C.c_void_p, _u8p, _u32p, C.c_uint64,
                            C.c_int, C.c_int, C.c_int, C.c_int, _tp(dtype))
        self.h = new()

    def decode(self, blob, sizes, n, exp, s, num, level):
        out = np.zeros(n, self.dtype)
        rc = self._dec(self.h, np.ascontiguousarray(blob, np.uint8), np.ascontiguousarray(sizes, np.uint32), n, exp,
                       s, num, level, out)
        if rc != 0:
            raise ValueError("grouped decode failed (%d)" % rc)
        return out

    def __del__(self):
        try:
            self._free(self.h)
        except Exception:
            pass


class _PerBitState:
    def __init__(self, lib, dtype):
        self.dtype, sfx, pre = np.dtype(dtype), _sfx(dtype), lib.prefix
        if pre == "ref":
            new, free, dec = "ref_pb_new_", "ref_pb_free_", "ref_pb_decode_"
        else:
            new, free, dec = "or_pb_state_new_", "or_pb_state_free_", "or_pb_decode_"
        self._free = lib._fn(free + sfx, None, C.c_void_p)
        self._dec = lib._fn(dec + sfx, C.c_int, C.c_void_p, _u8p, _u32p, C.c_uint64, C.c_int, C.c_int, C.c_int,
                            C.c_int, _tp(dtype))
        self.h = lib._fn(new + sfx, C.c_void_p)()

    def decode(self, blob, sizes, n, exp, s, num, level):
        out = np.zeros(n, self.dtype)
        self._dec(self.h, np.ascontiguousarray(blob, np.uint8), np.ascontiguousarray(sizes, np.uint32), n, exp, s, num,
                  level, out)
        return out

    def __del__(self):
        try:
            self._free(self.h)
        except Exception:
            pass


class Reference(Oracle):
    """The reference's own components, compiled by oracle/build_oracle.build_ref."""

    prefix = "ref"

    def _setup(self):
        pass

    def encode(self, kind, data, exp, B, collect=False):
        return Oracle.encode(self, kind, data, exp, B, collect)

    def level_dims_elements(self, dims, L, dtype=np.float32):
        d = np.asarray(dims, np.uint32)
        out = np.zeros((L + 1) * len(d), np.uint32)
        el = np.zeros(L + 1, np.uint32)
        f = self._fn("ref_level_dims_" + _sfx(dtype), None, C.c_int, _u32p, C.c_int, _u32p, _u32p)
        f(len(d), d, L, out, el)
        return out.reshape(L + 1, len(d)), el

    def decoder(self, kind, dtype):
        return _RefDecoder(self, kind, dtype)

    def interleave(self, data, dims, fine, coarse):
        s = _sfx(data.dtype)
        f = self._fn("ref_interleave_" + s, None, _tp(data.dtype), C.c_int, _u32p, _u32p, _u32p, _tp(data.dtype))
        fine = np.asarray(fine, np.uint32); coarse = np.asarray(coarse, np.uint32)
        n = int(np.prod(fine.astype(np.int64))) - int(np.prod(coarse.astype(np.int64)))
        buf = np.zeros(n, data.dtype)
        f(np.ascontiguousarray(data), len(dims), np.asarray(dims, np.uint32), fine, coarse, buf)
        return buf

    def max_collect(self, bound, B, dtype):
        f = self._fn("ref_max_collect_" + _sfx(dtype), None, _ct(dtype), C.c_int, _f64p)
        out = np.zeros(B + 1, np.float64)
        f(bound, B, out)
        return out

    def sq_collect(self, data, B, maxv):
        f = self._fn("ref_sq_collect_" + _sfx(data.dtype), None, _tp(data.dtype), C.c_uint64, C.c_int,
                     _ct(data.dtype), _f64p)
        out = np.zeros(B + 1, np.float64)
        f(np.ascontiguousarray(data), len(data), B, maxv, out)
        return out

    def adaptive_compress(self, blob, sizes, latter=26):
        """The reference's AdaptiveLevelCompressor (zstd level 3) on one level's
        streams: (stopping index, sizes it leaves, zstd size of every stream)."""
        B = len(sizes)
        out = np.zeros(B, np.uint32)
        zs = np.zeros(B, np.uint32)
        f = self._fn("ref_adaptive_compress", C.c_int, _u8p, _u32p, C.c_int, C.c_int, _u32p, _u32p)
        stop = f(np.ascontiguousarray(blob, np.uint8), np.ascontiguousarray(sizes, np.uint32), B, int(latter), out, zs)
        return stop, out, zs

    def headline_step(self, field, L, B, tols, out=None):
        """One benchmark step on the reference's own classes (fp32, negabinary,
        encoder squared-error tables, NegaBinary greedy interpreter with
        L2ErrorEstimator_HB, hierarchical basis); tols are absolute squared
        tolerances. Returns the step's algorithmic bytes."""
        f = self._fn("ref_headline_step_f32", C.c_int64, _f32p, _u32p, C.c_int, C.c_int, C.c_int, _f64p, C.c_void_p)
        tols = np.ascontiguousarray(tols, np.float64)
        x = np.ascontiguousarray(field, np.float32)
        optr = out.ctypes.data_as(C.c_void_p) if out is not None else None
        r = f(x.ravel(), np.asarray(field.shape, np.uint32), int(L), int(B), len(tols), tols, optr)
        if r < 0:
            raise RuntimeError("reference step failed")
        return int(r)

    def composed(self, field, L, B, encoder, hierarchical, tols, workdir):
        dims = np.asarray(field.shape, np.uint32)
        dt = field.dtype
        tols = np.asarray(tols, np.float64)
        outs = np.zeros((len(tols), field.size), dt)
        ret = np.zeros(len(tols), np.uint64)
        if encoder == "perbit":
            if not hierarchical:
                raise ValueError("the reference's PerBit drivers use the hierarchical basis")
            f = self._fn("ref_composed_pb_" + _sfx(dt), C.c_int, _tp(dt), C.c_int, _u32p, C.c_int, C.c_int,
                         C.c_char_p, C.c_int, _f64p, _tp(dt), np.ctypeslib.ndpointer(np.uint64))
            rc = f(np.ascontiguousarray(field).ravel(), len(dims), dims, L, B, workdir.encode(), len(tols), tols,
                   outs, ret)
            if rc != 0:
                raise RuntimeError("reference composed round trip failed")
            return outs.reshape((len(tols),) + field.shape), ret
        f = self._fn("ref_composed_" + _sfx(dt), C.c_int, _tp(dt), C.c_int, _u32p, C.c_int, C.c_int, C.c_int,
                     C.c_int, C.c_char_p, C.c_int, _f64p, _tp(dt), np.ctypeslib.ndpointer(np.uint64))
        rc = f(np.ascontiguousarray(field).ravel(), len(dims), dims, L, B, ENCODERS[encoder], int(hierarchical),
               workdir.encode(), len(tols), tols, outs, ret)
        if rc != 0:
            raise RuntimeError("reference composed round trip failed")
        return outs.reshape((len(tols),) + field.shape), ret

    def composed_zstd(self, field, L, B, encoder, latter, tols, workdir):
        """The round trip above with the reference's zstd stage,
        AdaptiveLevelCompressor(latter) (fp32, hierarchical basis): writes
        workdir/metadata.bin and workdir/level_<l>.bin as a stock refactor
        does, and returns the reference reconstructor's outputs and retrieved
        sizes for the tolerances (SignExclude greedy, MaxErrorEstimatorHB)."""
        dims = np.asarray(field.shape, np.uint32)
        tols = np.asarray(tols, np.float64)
        outs = np.zeros((len(tols), field.size), np.float32)
        ret = np.zeros(len(tols), np.uint64)
        f = self._fn("ref_composed_zstd_f32", C.c_int, _tp(np.float32), C.c_int, _u32p, C.c_int, C.c_int, C.c_int,
                     C.c_int, C.c_char_p, C.c_int, _f64p, _tp(np.float32), np.ctypeslib.ndpointer(np.uint64))
        rc = f(np.ascontiguousarray(field, np.float32).ravel(), len(dims), dims, L, B, ENCODERS[encoder], int(latter),
               workdir.encode(), len(tols), tols, outs, ret)
        if rc != 0:
            raise RuntimeError("reference composed round trip failed")
        return outs.reshape((len(tols),) + field.shape), ret


class _RefDecoder:
    def __init__(self, lib, kind, dtype):
        self.lib, self.kind, self.dtype, self.sfx = lib, kind, np.dtype(dtype), _sfx(dtype)
        k = "gr" if kind == "grouped" else "nb"
        self.h = lib._fn("ref_%s_new_%s" % (k, self.sfx), C.c_void_p)()
        self._free = lib._fn("ref_%s_free_%s" % (k, self.sfx), None, C.c_void_p)
        self._dec = lib._fn("ref_decode_" + self.sfx, C.c_int, C.c_void_p, C.c_int, _u8p, _u32p, C.c_uint64, C.c_int,
                            C.c_int, C.c_int, C.c_int, _tp(dtype))

    def decode(self, blob, sizes, n, exp, s, num, level):
        out = np.zeros(n, self.dtype)
        self._dec(self.h, int(self.kind == "grouped"), np.ascontiguousarray(blob, np.uint8),
                  np.ascontiguousarray(sizes, np.uint32), n, exp, s, num, level, out)
        return out

    def __del__(self):
        try:
            self._free(self.h)
        except Exception:
            pass


_oracle = None
_ref = None


def oracle():
    """The oracle restatement, built on first use."""
    global _oracle
    if _oracle is None:
        _oracle = Oracle(build_oracle())
    return _oracle


def reference():
    """The reference harness, or None where it cannot be built or loaded."""
    global _ref
    if _ref is None:
        path = build_ref()
        if path is None or not os.path.exists(path):
            return None
        try:
            _ref = Reference(path)
        except OSError:
            return None
    return _ref
