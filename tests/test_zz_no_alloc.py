"""prodm_collect_squared_noalloc (the squared error collector that allocates
nothing, for callers that cannot allocate device memory) against
prodm_collect_squared, both called through the C ABI, on two calls in a row.
The file is named to be collected last and also runs alone."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ERR_RTOL = 1e-12   # the tolerance of the other squared-error table tests
F32, F64 = 0, 1


def _lib():
    from prodm_gb300 import _lib as L
    return L.load()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _existing(lib, x, B, maxv):
    out = torch.zeros(B + 1, dtype=torch.float64, device="cuda")
    dt = F64 if x.dtype == torch.float64 else F32
    rc = lib.prodm_collect_squared(dt, C.c_void_p(x.data_ptr()), x.numel(), B, maxv, C.c_void_p(out.data_ptr()),
                                   None, 0, _stream())
    assert rc == 0, lib.prodm_last_error_string()
    return out


def _noalloc(lib, x, B, maxv):
    out = torch.full((B + 1,), float("nan"), dtype=torch.float64, device="cuda")
    dt = F64 if x.dtype == torch.float64 else F32
    rc = lib.prodm_collect_squared_noalloc(dt, C.c_void_p(x.data_ptr()), x.numel(), B, maxv,
                                           C.c_void_p(out.data_ptr()), _stream())
    assert rc == 0, lib.prodm_last_error_string()
    return out


def _case(seed, n, dtype):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    x = (x * torch.exp(2.0 * torch.randn(n, dtype=torch.float64, device="cuda", generator=g))).to(dtype)
    x[::97] = 0
    return x, float(x.abs().max())


def test_noalloc_matches_collect_squared_two_calls_in_a_row():
    lib = _lib()
    # first call: the largest table (fp64, 64 bitplanes); second call: a
    # smaller fp32 table over a different field, which must not see the
    # first call's partial tables left in the shared scratch
    x1, m1 = _case(1, (1 << 22) + 7, torch.float64)
    x2, m2 = _case(2, (1 << 21) + 333, torch.float32)
    a1 = _noalloc(lib, x1, 64, m1)
    a2 = _noalloc(lib, x2, 23, m2)
    torch.cuda.synchronize()
    r1 = _existing(lib, x1, 64, m1)
    r2 = _existing(lib, x2, 23, m2)
    torch.cuda.synchronize()
    for got, ref in ((a1, r1), (a2, r2)):
        got, ref = got.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(got))
        np.testing.assert_allclose(got, ref, rtol=ERR_RTOL, atol=1e-30)


def test_noalloc_small_inputs_and_limits():
    lib = _lib()
    for n, B in ((1, 1), (31, 32), (1000, 8)):
        x, m = _case(n, n, torch.float32)
        got = _noalloc(lib, x, B, m).cpu().numpy()
        ref = _existing(lib, x, B, m).cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=ERR_RTOL, atol=1e-30)
    # beyond the fixed scratch: rejected on the host with a message
    x, m = _case(3, 100, torch.float32)
    out = torch.zeros(70, dtype=torch.float64, device="cuda")
    rc = lib.prodm_collect_squared_noalloc(F32, C.c_void_p(x.data_ptr()), x.numel(), 33, m,
                                           C.c_void_p(out.data_ptr()), _stream())
    assert rc == 1 and b"num_bitplanes" in lib.prodm_last_error_string()
    x64 = x.double()
    rc = lib.prodm_collect_squared_noalloc(F64, C.c_void_p(x64.data_ptr()), x64.numel(), 65, m,
                                           C.c_void_p(out.data_ptr()), _stream())
    assert rc == 1 and b"num_bitplanes" in lib.prodm_last_error_string()


def test_noalloc_allocates_no_device_memory():
    # warmed up (address looked up, torch's own tensors allocated), then two
    # more calls leave the device's free memory exactly as it was
    lib = _lib()
    x, m = _case(5, (1 << 20) + 3, torch.float64)
    out = torch.zeros(65, dtype=torch.float64, device="cuda")
    st = _stream()

    def call():
        rc = lib.prodm_collect_squared_noalloc(F64, C.c_void_p(x.data_ptr()), x.numel(), 64, m,
                                               C.c_void_p(out.data_ptr()), st)
        assert rc == 0, lib.prodm_last_error_string()

    call()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    call()
    call()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
