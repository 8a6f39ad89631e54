"""Python host API over the C ABI (device memory and streams come from torch).

Component functions mirror the reference's plugin concepts (decompose /
recompose, interleave / reposition, encode / progressive_decode, error
collectors, size interpreters); ``MDRField`` is the device-resident composed
refactor / reconstructor. All arrays are torch CUDA tensors; nothing here
computes on the CPU.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import BASIS, COLLECT, ENC, EST, INTERP, call, load

_DT = {torch.float32: _lib.F32, torch.float64: _lib.F64}


def _dtype(t):
    try:
        return _DT[t.dtype]
    except KeyError:
        raise TypeError("only float32 and float64 tensors are supported")


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _u32(seq):
    a = (C.c_uint32 * len(seq))(*[int(x) for x in seq])
    return a


def _ptr(t):
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return C.c_void_p(t.data_ptr())


def max_level(dims):
    out = C.c_int()
    call("prodm_max_level", len(dims), _u32(dims), C.byref(out))
    return out.value


def level_dims(dims, L):
    nd = len(dims)
    out = (C.c_uint32 * ((L + 1) * nd))()
    el = (C.c_uint64 * (L + 1))()
    call("prodm_level_dims", nd, _u32(dims), L, out, el)
    return np.array(out[:], np.uint32).reshape(L + 1, nd), np.array(el[:], np.uint64)


# ---------------------------------------------------------------------------
# components
# ---------------------------------------------------------------------------
def decompose(data, target_level, basis="hierarchical", dims=None, stream=None, workspace=None):
    """In-place MGARD decomposition of a CUDA tensor (reference layout)."""
    dims = list(dims or data.shape)
    ws, wsb = (None, 0) if workspace is None else (_ptr(workspace), workspace.numel() * workspace.element_size())
    call("prodm_decompose", _dtype(data), _ptr(data), len(dims), _u32(dims), target_level, None, BASIS[basis], ws, wsb,
         _stream(stream))
    return data


def recompose(data, target_level, basis="hierarchical", dims=None, stream=None, workspace=None):
    dims = list(dims or data.shape)
    ws, wsb = (None, 0) if workspace is None else (_ptr(workspace), workspace.numel() * workspace.element_size())
    call("prodm_recompose", _dtype(data), _ptr(data), len(dims), _u32(dims), target_level, None, BASIS[basis], ws, wsb,
         _stream(stream))
    return data


def interleave(data, fine, coarse, stream=None):
    n = int(np.prod(fine, dtype=np.int64)) - int(np.prod(coarse, dtype=np.int64))
    buf = torch.empty(n, dtype=data.dtype, device=data.device)
    dims = list(data.shape)
    call("prodm_interleave", _dtype(data), _ptr(data), len(dims), _u32(dims), _u32(fine), _u32(coarse), _ptr(buf),
         None, _stream(stream))
    return buf


def reposition(buf, data, fine, coarse, stream=None):
    dims = list(data.shape)
    call("prodm_reposition", _dtype(buf), _ptr(buf), len(dims), _u32(dims), _u32(fine), _u32(coarse), _ptr(data),
         None, _stream(stream))
    return data


def encode(kind, data, exp, num_bitplanes, collect=False, stream=None):
    """Returns (blob uint8 tensor cut to size, sizes numpy[B], errors numpy[B+1] or None)."""
    n = data.numel()
    bound = C.c_uint64()
    call("prodm_encode_bound", ENC[kind], _dtype(data), n, num_bitplanes, C.byref(bound))
    blob = torch.empty(bound.value + 16, dtype=torch.uint8, device=data.device)
    sizes = torch.empty(num_bitplanes, dtype=torch.int32, device=data.device)
    errs = torch.empty(num_bitplanes + 1, dtype=torch.float64, device=data.device) if collect else None
    call("prodm_encode", ENC[kind], _dtype(data), _ptr(data), n, int(exp), num_bitplanes, _ptr(blob), bound.value,
         _ptr(sizes), _ptr(errs) if collect else None, None, 0, _stream(stream))
    sz = sizes.cpu().numpy().view(np.uint32).copy()
    total = int(sz.astype(np.int64).sum())
    return blob[:total], sz, (errs.cpu().numpy() if collect else None)


def compress_level(blob, sizes, latter_index=26, stream=None):
    """The lossless stage on one level's streams (device uint8 tensor, sizes):
    returns (stored streams as a device uint8 tensor, their sizes, stopping index)."""
    B = len(sizes)
    hs = (C.c_uint32 * B)(*[int(x) for x in sizes])
    bound = C.c_uint64()
    call("prodm_lossless_compress_bound", hs, B, C.byref(bound))
    out = torch.empty(max(bound.value, 1), dtype=torch.uint8, device=blob.device)
    osz = (C.c_uint32 * B)()
    stop = C.c_int()
    call("prodm_lossless_compress_level", _ptr(blob), hs, B, int(latter_index), _ptr(out), bound.value, osz,
         C.byref(stop), _stream(stream))
    sz = np.array(osz[:], np.uint32)
    return out[:int(sz.astype(np.int64).sum())], sz, stop.value


def decompress_level(blob, sizes, start, num, stopping_index, latter_index=26, raw_capacity=None, stream=None):
    """Stored streams of planes [start, start+num) -> (raw streams concatenated, raw sizes)."""
    hs = (C.c_uint32 * max(num, 1))(*[int(x) for x in sizes[:num]])
    cap = int(raw_capacity) if raw_capacity is not None else 64 * max(int(blob.numel()), 1)
    out = torch.empty(max(cap, 1), dtype=torch.uint8, device=blob.device)
    rsz = (C.c_uint32 * max(num, 1))()
    call("prodm_lossless_decompress_level", _ptr(blob), hs, int(start), int(num), int(stopping_index),
         int(latter_index), _ptr(out), cap, rsz, _stream(stream))
    r = np.array(rsz[:num], np.uint32)
    return out[:int(r.astype(np.int64).sum())], r


class ProgressiveDecoder:
    """Stateful decoder (grouped state per level), BitplaneEncoderInterface::progressive_decode."""

    def __init__(self, kind, dtype):
        self.kind, self.dtype = kind, dtype
        self.h = C.c_void_p()
        call("prodm_decoder_create", C.byref(self.h), ENC[kind], _DT[dtype])

    def decode(self, blob, sizes, n, exp, start, num, level, total_bitplanes, stream=None):
        out = torch.empty(n, dtype=self.dtype, device="cuda")
        hs = (C.c_uint32 * max(1, num))(*[int(x) for x in sizes[:num]])
        call("prodm_progressive_decode", self.h, _ptr(blob) if num else None, hs, n, int(exp), start, num, level,
             total_bitplanes, _ptr(out), _stream(stream))
        return out

    def __del__(self):
        try:
            if self.h:
                load().prodm_decoder_destroy(self.h)
        except Exception:
            pass


def collect_max(bound, num_bitplanes, dtype=torch.float32):
    out = (C.c_double * (num_bitplanes + 1))()
    call("prodm_collect_max", _DT[dtype], float(bound), num_bitplanes, out)
    return np.array(out[:])


def collect_squared(data, num_bitplanes, max_level_error, stream=None):
    out = torch.empty(num_bitplanes + 1, dtype=torch.float64, device=data.device)
    call("prodm_collect_squared", _dtype(data), _ptr(data), data.numel(), num_bitplanes, float(max_level_error),
         _ptr(out), None, 0, _stream(stream))
    return out.cpu().numpy()


def recompose_packed(coef, shape, target_level, out=None, stream=None, basis="hierarchical"):
    """Packed level coefficients (the layout of MDRField.coefficients()) ->
    natural-order field of `shape` (hierarchical or orthogonal basis)."""
    shape = tuple(int(n) for n in shape)
    if out is None:
        out = torch.empty(shape, dtype=coef.dtype, device=coef.device)
    dims = _u32(shape)
    call("prodm_recompose_packed_basis", _dtype(coef), BASIS[basis], _ptr(coef), len(shape), dims, int(target_level),
         _ptr(out), None, 0, _stream(stream))
    return out


def recompose_adjoint(grad, target_level, out=None, stream=None, basis="hierarchical"):
    """Transpose of recompose_packed: gradient with respect to the natural-order
    field -> gradient with respect to the packed level coefficients."""
    shape = tuple(grad.shape)
    if out is None:
        out = torch.empty(grad.numel(), dtype=grad.dtype, device=grad.device)
    dims = _u32(shape)
    call("prodm_recompose_adjoint_basis", _dtype(grad), BASIS[basis], _ptr(grad.contiguous()), len(shape), dims,
         int(target_level), _ptr(out), None, 0, _stream(stream))
    return out


def _same_fields(ts):
    """All given device fields contiguous, of one dtype and one element count
    (the kernels index them with one flat index)."""
    ts = [t for t in ts if t is not None]
    if not ts:
        raise ValueError("no fields given")
    for t in ts:
        if not t.is_contiguous():
            raise ValueError("fields must be contiguous")
        if t.dtype != ts[0].dtype or t.numel() != ts[0].numel():
            raise ValueError("fields must share dtype and element count")
    return ts[0]


def qoi_ge_values(vx, vy, vz, p, d, stream=None):
    """V_TOT, T, C, Mach, PT, mu of fp64 device fields (six new tensors)."""
    _same_fields([vx, vy, vz, p, d])
    outs = [torch.empty_like(vx) for _ in range(6)]
    call("prodm_qoi_ge_values", _dtype(vx), _ptr(vx), _ptr(vy), _ptr(vz), _ptr(p), _ptr(d), vx.numel(),
         *[_ptr(o) for o in outs], _stream(stream))
    return outs


def qoi_ge_bounds(V=None, ebs_v=(0.0, 0.0, 0.0), P=None, D=None, eb_p=0.0, eb_d=0.0, stream=None):
    """Pointwise error estimates of V_TOT (from V = [vx, vy, vz]) and of T
    (from P, D), fp64 device fields. Returns (bound_vtot, bound_t, maxima)."""
    ref = _same_fields(list(V if V is not None else []) + [P, D])
    n = ref.numel()
    bv = torch.empty_like(ref) if V is not None else None
    bt = torch.empty_like(ref) if P is not None else None
    mx = torch.empty(2, dtype=torch.float64, device=ref.device)
    nul = C.c_void_p(None)
    vp = [_ptr(v) for v in V] if V is not None else [nul, nul, nul]
    call("prodm_qoi_ge_bounds", _dtype(ref), *vp, _ptr(P) if P is not None else nul,
         _ptr(D) if D is not None else nul, n, *[float(e) for e in ebs_v], float(eb_p), float(eb_d),
         _ptr(bv) if bv is not None else nul, _ptr(bt) if bt is not None else nul, _ptr(mx), _stream(stream))
    return bv, bt, mx


def interpret(kind, estimator, sizes, errors, tolerance, index, ndims=3, target_level=None, s=0.0,
              dtype=torch.float32, stream=None):
    """Device greedy interpreter. sizes [nl,B] (uint32), errors [nl,B+1]; returns (index, retrieve_sizes)."""
    sizes = np.ascontiguousarray(sizes, np.uint32)
    nl, B = sizes.shape
    L = nl - 1 if target_level is None else target_level
    dsz = torch.from_numpy(sizes.view(np.int32)).cuda()
    derr = torch.from_numpy(np.ascontiguousarray(errors, np.float64)).cuda()
    didx = torch.from_numpy(np.ascontiguousarray(index, np.uint8).copy()).cuda()
    drsz = torch.zeros(nl, dtype=torch.int32, device="cuda")
    call("prodm_interpret", INTERP[kind], EST[estimator], _DT[dtype], ndims, L, float(s), nl, B, _ptr(dsz), _ptr(derr),
         float(tolerance), _ptr(didx), _ptr(drsz), _stream(stream))
    return didx.cpu().numpy(), drsz.cpu().numpy().view(np.uint32)


# ---------------------------------------------------------------------------
# device-resident composed refactor / reconstructor
# ---------------------------------------------------------------------------
class MDRField:
    """One field configuration: refactor on the device, retrieve progressively.

    Mirrors ComposedRefactor::refactor (ComposedRefactor.hpp:21-141) and
    ComposedReconstructor::progressive_reconstruct (ComposedReconstructor.hpp:
    106-122) with all state resident in HBM.
    """

    def __init__(self, shape, dtype=torch.float32, target_level=None, num_bitplanes=32, encoder="negabinary",
                 basis="hierarchical", collector="max"):
        self.shape = tuple(int(x) for x in shape)
        self.dtype = dtype
        if target_level is None:
            target_level = max_level(self.shape)
        self.L, self.B = int(target_level), int(num_bitplanes)
        self.encoder, self.basis, self.collector = encoder, basis, collector
        cfg = _lib.prodm_config()
        cfg.dtype = _DT[dtype]
        cfg.ndims = len(self.shape)
        for i, d in enumerate(self.shape):
            cfg.dims[i] = d
        cfg.target_level = self.L
        cfg.num_bitplanes = self.B
        cfg.encoder = ENC[encoder]
        cfg.basis = BASIS[basis]
        cfg.collector = COLLECT[collector]
        self.h = C.c_void_p()
        call("prodm_mdr_create", C.byref(self.h), C.byref(cfg))
        self.level_dims, self.level_elements = level_dims(self.shape, self.L)

    def refactor(self, field, stream=None):
        if field.dtype != self.dtype or tuple(field.shape) != self.shape or not field.is_contiguous():
            raise ValueError("field must be a contiguous %s tensor of shape %s" % (self.dtype, self.shape))
        call("prodm_mdr_refactor", self.h, _ptr(field), _stream(stream))

    def level_info(self, stream=None):
        nl, B = self.L + 1, self.B
        sizes = (C.c_uint32 * (nl * B))()
        bounds = (C.c_double * nl)()
        errs = (C.c_double * (nl * (B + 1)))()
        call("prodm_mdr_level_info", self.h, sizes, bounds, errs, _stream(stream))
        return (np.array(sizes[:], np.uint32).reshape(nl, B), np.array(bounds[:]),
                np.array(errs[:]).reshape(nl, B + 1))

    def metadata(self, stream=None):
        n = C.c_size_t()
        call("prodm_mdr_metadata", self.h, None, 0, C.byref(n), _stream(stream))
        buf = (C.c_uint8 * n.value)()
        call("prodm_mdr_metadata", self.h, buf, n.value, C.byref(n), _stream(stream))
        return bytes(buf)

    def export_level(self, level, stream=None):
        n = C.c_uint64()
        call("prodm_mdr_export_level", self.h, level, None, 0, 1, C.byref(n), _stream(stream))
        buf = np.zeros(n.value, np.uint8)
        call("prodm_mdr_export_level", self.h, level, C.c_void_p(buf.ctypes.data), n.value, 1, C.byref(n),
             _stream(stream))
        return buf

    def export_level_device(self, level, stream=None):
        """The level file's bytes as a device uint8 tensor."""
        n = C.c_uint64()
        call("prodm_mdr_export_level", self.h, level, None, 0, 0, C.byref(n), _stream(stream))
        buf = torch.empty(max(n.value, 1), dtype=torch.uint8, device="cuda")
        call("prodm_mdr_export_level", self.h, level, _ptr(buf), n.value, 0, C.byref(n), _stream(stream))
        return buf[:n.value]

    def export_level_into(self, level, out, stream=None):
        """The level file's bytes into `out` (a uint8 tensor: CUDA, or pinned
        host memory filled asynchronously in the stream's order); returns the
        byte count."""
        if out.dtype != torch.uint8 or not out.is_contiguous():
            raise ValueError("expected a contiguous uint8 tensor")
        if not out.is_cuda and not out.is_pinned():
            raise ValueError("host output must be pinned memory")
        n = C.c_uint64()
        call("prodm_mdr_export_level", self.h, level, C.c_void_p(out.data_ptr()), out.numel(),
             0 if out.is_cuda else 2, C.byref(n), _stream(stream))
        return n.value

    def export_level_range_into(self, level, offset, out, stream=None):
        """Bytes [offset, offset + out.numel()) of the level file into `out` (a
        uint8 tensor: CUDA, or pinned host memory filled asynchronously in the
        stream's order)."""
        if out.dtype != torch.uint8 or not out.is_contiguous():
            raise ValueError("expected a contiguous uint8 tensor")
        if not out.is_cuda and out.numel() and not out.is_pinned():
            raise ValueError("host output must be pinned memory")
        call("prodm_mdr_export_level_range", self.h, level, int(offset), out.numel(),
             C.c_void_p(out.data_ptr()) if out.numel() else None, 0 if out.is_cuda else 2, _stream(stream))

    def set_lossless(self, latter_index=26, stream=None):
        """Lossless stage on (latter_index >= 0, the reference's default 26) or off (None / < 0)."""
        call("prodm_mdr_set_lossless", self.h, -1 if latter_index is None else int(latter_index), _stream(stream))

    def set_zstd_latter(self, latter_index=26):
        """Latter index of the reference's AdaptiveLevelCompressor that wrote
        zstd level files (its constructor argument); call before load_metadata."""
        call("prodm_mdr_set_zstd_latter", self.h, int(latter_index))

    def retrieve(self, tolerance, out=None, interpreter="sign_exclude", estimator="max_hb", s=0.0, stream=None):
        if out is None:
            out = torch.empty(self.shape, dtype=self.dtype, device="cuda")
        call("prodm_mdr_retrieve", self.h, float(tolerance), INTERP[interpreter], EST[estimator], float(s), _ptr(out),
             _stream(stream))
        return out

    def interpret(self, tolerance, interpreter="sign_exclude", estimator="max_hb", s=0.0, stream=None):
        call("prodm_mdr_interpret", self.h, float(tolerance), INTERP[interpreter], EST[estimator], float(s),
             _stream(stream))

    def reconstruct(self, out=None, stream=None):
        if out is None:
            out = torch.empty(self.shape, dtype=self.dtype, device="cuda")
        call("prodm_mdr_reconstruct", self.h, _ptr(out), _stream(stream))
        return out

    def load_metadata(self, meta, stream=None):
        buf = (C.c_uint8 * len(meta)).from_buffer_copy(meta)
        call("prodm_mdr_load_metadata", self.h, buf, len(meta), _stream(stream))

    def load_level(self, level, src, offset=0, stream=None):
        """src: numpy uint8 array (host) or torch uint8 tensor (host pinned or device)."""
        if isinstance(src, np.ndarray):
            src = np.ascontiguousarray(src, np.uint8)
            ptr, host, n = C.c_void_p(src.ctypes.data), 1, src.nbytes
        else:
            ptr, host, n = C.c_void_p(src.data_ptr()), 0 if src.is_cuda else 1, src.numel()
        call("prodm_mdr_load_level", self.h, level, ptr, int(offset), int(n), host, _stream(stream))

    def load_level_file(self, level, path, file_offset=0, level_offset=0, nbytes=None, stream=None):
        """Bytes of a level file straight into device memory (cuFile or pinned staging)."""
        import os
        if nbytes is None:
            nbytes = os.path.getsize(path) - int(file_offset)
        call("prodm_mdr_load_level_file", self.h, level, str(path).encode(), int(file_offset), int(level_offset),
             int(nbytes), _stream(stream))

    def write_level_file(self, level, path, stream=None):
        call("prodm_mdr_write_level_file", self.h, level, str(path).encode(), _stream(stream))

    def file_read_mode(self):
        """1: cuFile (GPUDirect Storage), 0: pinned staging, -1: no file read yet."""
        m = C.c_int()
        call("prodm_mdr_file_read_mode", self.h, C.byref(m))
        return m.value

    def retrieve_planes(self, index, out=None, stream=None):
        if out is None:
            out = torch.empty(self.shape, dtype=self.dtype, device="cuda")
        idx = (C.c_uint8 * (self.L + 1))(*[int(x) for x in index])
        call("prodm_mdr_retrieve_planes", self.h, idx, _ptr(out), _stream(stream))
        return out

    def index(self, stream=None):
        idx = (C.c_uint8 * (self.L + 1))()
        call("prodm_mdr_get_index", self.h, idx, _stream(stream))
        return np.array(idx[:], np.uint8)

    def reset(self, stream=None):
        call("prodm_mdr_reset_retrieval", self.h, _stream(stream))

    def status(self, stream=None):
        """Raises ProdmError (PRODM_ETIMEOUT) when a bounded wait of an earlier
        retrieval kernel gave up; the status is cleared once reported."""
        call("prodm_mdr_status", self.h, _stream(stream))

    def coefficients(self, stream=None):
        """Packed level coefficients of the last refactor (a device copy)."""
        n = int(self.level_elements.astype(np.int64).sum())
        t = torch.empty(n, dtype=self.dtype, device="cuda")
        call("prodm_mdr_coefficients", self.h, _ptr(t), _stream(stream))
        return t

    def retrieved_bytes(self, index=None):
        sizes, _, _ = self.level_info()
        idx = self.index() if index is None else index
        return int(sum(int(sizes[l, :idx[l]].astype(np.int64).sum()) for l in range(self.L + 1)))

    def set_timing(self, enable=True):
        call("prodm_mdr_set_timing", self.h, int(enable))

    def stage_times(self):
        """{(kind, level): (total_ms, count)} for stages timed since set_timing(True)."""
        ms = (C.c_double * 85)()
        cnt = (C.c_uint32 * 85)()
        call("prodm_mdr_stage_times", self.h, ms, cnt)
        kinds = ("decompose", "encode", "interpret", "decode", "recompose")
        return {(kinds[i // 17], i % 17): (ms[i], cnt[i]) for i in range(85) if cnt[i]}

    def close(self):
        if self.h:
            load().prodm_mdr_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launch_count():
    out = C.c_uint64()
    call("prodm_kernel_launch_count", C.byref(out))
    return out.value


def debug_tile_wait(extra_tx_bytes=0, wait_cycles=0):
    """Test hook for the fused kernel's timeout path (prodm_debug_tile_wait);
    (0, 0) restores normal operation."""
    call("prodm_debug_tile_wait", int(extra_tx_bytes), int(wait_cycles))


class MDRBatch:
    """Many fp32 fields refactored / retrieved together (one launch per stage).

    fields: list of contiguous fp32 CUDA tensors (kept referenced: their
    device pointers are bound into the launch tables).
    """

    def __init__(self, fields, levels=None, num_bitplanes=32):
        self.fields = list(fields)
        self.outs = [torch.empty_like(f) for f in self.fields]
        n = len(self.fields)
        cfgs = (_lib.prodm_config * n)()
        self.levels = []
        for i, f in enumerate(self.fields):
            if f.dtype != torch.float32 or not f.is_contiguous() or not f.is_cuda:
                raise ValueError("batched fields must be contiguous fp32 CUDA tensors")
            L = max_level(f.shape) if levels is None else int(levels[i])
            self.levels.append(L)
            c = cfgs[i]
            c.dtype = _lib.F32
            c.ndims = f.dim()
            for d, v in enumerate(f.shape):
                c.dims[d] = v
            c.target_level = L
            c.num_bitplanes = num_bitplanes
            c.encoder = ENC["negabinary"]
            c.basis = BASIS["hierarchical"]
            c.collector = COLLECT["max"]
        self.B = num_bitplanes
        self.h = C.c_void_p()
        call("prodm_batch_create", C.byref(self.h), n, cfgs)
        fp = (C.c_void_p * n)(*[f.data_ptr() for f in self.fields])
        op = (C.c_void_p * n)(*[o.data_ptr() for o in self.outs])
        call("prodm_batch_bind", self.h, fp, op)

    def set_launch(self, threads_per_cta, ctas_per_sm):
        call("prodm_batch_set_launch", self.h, int(threads_per_cta), int(ctas_per_sm))

    STAGES = {"decompose": 0, "encode": 1, "recompose": 2, "fused": 3}

    def set_stage_launch(self, stage, threads_per_cta, ctas_per_sm):
        """stage: "decompose", "encode", "recompose" or "fused" (the finest
        levels, decoded inside their recomposition)."""
        call("prodm_batch_set_stage_launch", self.h, self.STAGES[stage], int(threads_per_cta), int(ctas_per_sm))

    def set_fused_unit(self, values_per_unit):
        """Tile shape of the fused finest levels: about this many values per
        unit of consecutive fine rows (rebuilds the segment tables)."""
        call("prodm_batch_set_fused_unit", self.h, int(values_per_unit))

    def refactor(self, stream=None):
        call("prodm_batch_refactor", self.h, _stream(stream))

    def set_tolerances(self, tols, stream=None):
        arr = (C.c_double * len(self.fields))(*[float(t) for t in tols])
        call("prodm_batch_set_tolerances", self.h, arr, _stream(stream))

    def retrieve(self, interpreter="negabinary", estimator="max_hb", s=0.0, stream=None):
        call("prodm_batch_retrieve", self.h, INTERP[interpreter], EST[estimator], float(s), _stream(stream))
        return self.outs

    def reset(self, stream=None):
        call("prodm_batch_reset", self.h, _stream(stream))

    def status(self, stream=None):
        """Raises ProdmError when a fused kernel reported an error since the
        last call (PRODM_ETIMEOUT: a wait for plane tiles gave up)."""
        call("prodm_batch_status", self.h, _stream(stream))

    def field_info(self, i, stream=None):
        nl = self.levels[i] + 1
        idx = (C.c_uint8 * nl)()
        sz = (C.c_uint32 * (nl * self.B))()
        bd = (C.c_double * nl)()
        call("prodm_batch_field_info", self.h, i, idx, sz, bd, _stream(stream))
        return np.array(idx[:], np.uint8), np.array(sz[:], np.uint32).reshape(nl, self.B), np.array(bd[:])

    def export_level(self, i, level, stream=None):
        n = C.c_uint64()
        call("prodm_batch_export_level", self.h, i, level, None, 0, 1, C.byref(n), _stream(stream))
        buf = np.zeros(n.value, np.uint8)
        call("prodm_batch_export_level", self.h, i, level, C.c_void_p(buf.ctypes.data), n.value, 1, C.byref(n),
             _stream(stream))
        return buf

    def close(self):
        if self.h:
            load().prodm_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
