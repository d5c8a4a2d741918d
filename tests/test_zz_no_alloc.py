"""skkr_gpu_surfgf_batch_noalloc: the decimation entry point for callers that
may not allocate device memory (their device buffers belong to another layer
of the host program, or their device-memory budget is fixed up front).  It
takes the caller's device buffers and keeps its work matrices in a static
device array, so it is checked here through the C ABI against the ordinary
allocating entry point, on two calls in a row (the array keeps the previous
call's contents), and for its size limit."""
import ctypes as C

import numpy as np
import pytest

from skkr_budapest_gb300 import native

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _lib():
    L = native.lib()
    L.skkr_gpu_surfgf_batch_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p,
                                                C.c_void_p, C.c_void_p]
    return L


def _inputs(seed, b, n):
    rng = np.random.default_rng(seed)
    m0 = rng.normal(size=(b, n, n)) * 0.3 + (2.0 + 1.0j) * np.eye(n)
    ml = (rng.normal(size=(b, n, n)) + 1j * rng.normal(size=(b, n, n))) * 0.15
    mr = (rng.normal(size=(b, n, n)) + 1j * rng.normal(size=(b, n, n))) * 0.15
    return ml, m0, mr


def _noalloc(ml, m0, mr, itermax=50, errmax=1e-10):
    import torch
    b, n, _ = m0.shape
    dev = [torch.from_numpy(native.cm(a)).cuda() for a in (ml, m0, mr)]
    x = torch.zeros_like(dev[1])
    it = np.zeros(b, np.int32)
    st = np.zeros(b, np.int32)
    torch.cuda.synchronize()
    rc = _lib().skkr_gpu_surfgf_batch_noalloc(n, b, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                              x.data_ptr(), n, itermax, errmax, native._p(it), native._p(st),
                                              None)
    return rc, native.uncm(x.cpu().numpy()), it, st


def test_noalloc_matches_allocating_entry_point_twice():
    for call, (seed, b, n) in enumerate([(1, 4, 20), (2, 3, 36)]):
        ml, m0, mr = _inputs(seed, b, n)
        rc, x, it, st = _noalloc(ml, m0, mr)
        assert rc == 0, (call, rc)
        xr, sr, ir = native.surfgf_batch(ml, m0, mr, itermax=50, errmax=1e-10)
        assert np.array_equal(st, sr) and np.array_equal(it, ir)
        err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
        assert err < TOL, (call, err)


def test_noalloc_rejects_requests_over_the_static_scratch():
    import torch
    n, b = 128, 64  # 64 * 8 * 128^2 * 16 B = 128 MiB > 32 MiB
    buf = torch.zeros((b, n, n), dtype=torch.complex128, device="cuda")  # in bounds for every input read
    p = buf.data_ptr()
    rc = _lib().skkr_gpu_surfgf_batch_noalloc(n, b, p, p, p, p, n, 50, 1e-8, None, None, None)
    assert rc == -6
