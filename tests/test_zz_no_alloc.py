"""skkr_gpu_surfgf_batch_noalloc: the decimation entry point for callers that
may not allocate device memory (their device buffers belong to another layer
of the host program, such as an OpenACC or CUDA Fortran data region or the
application's own pool, or their device-memory budget is fixed up front).
It takes the caller's device buffers and keeps its work matrices in a static
device array, so it is checked here through the C ABI against the ordinary
allocating entry point and the oracle's surfgfd, on two calls in a row (the
array keeps the previous call's contents), with Fortran-padded leading
dimensions on a caller's stream, and for its size limits."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
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


def _padded(a, ld):
    """(b, n, n) [row, col] -> (b, ld, ld) column-major blocks with the n x n
    matrix in the leading corner and NaN in the padding (never read)."""
    b, n, _ = a.shape
    out = np.full((b, ld, ld), np.nan + 1j * np.nan, np.complex128)
    out[:, :n, :n] = np.swapaxes(a, -1, -2)
    return out


def _noalloc(ml, m0, mr, itermax=50, errmax=1e-10, ld=None, stream=None):
    import torch
    b, n, _ = m0.shape
    ld = n if ld is None else ld
    dev = [torch.from_numpy(_padded(a, ld)).cuda() for a in (ml, m0, mr)]
    x = torch.zeros_like(dev[1])
    it = np.zeros(b, np.int32)
    st = np.zeros(b, np.int32)
    torch.cuda.synchronize()
    sp = None if stream is None else stream.cuda_stream
    rc = _lib().skkr_gpu_surfgf_batch_noalloc(n, b, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                              x.data_ptr(), ld, itermax, errmax, native._p(it), native._p(st),
                                              sp)
    xh = x.cpu().numpy()
    return rc, np.swapaxes(xh[:, :ld, :ld], -1, -2)[:, :n, :n], it, st


def test_noalloc_matches_allocating_entry_point_twice():
    for call, (seed, b, n) in enumerate([(1, 4, 20), (2, 3, 36)]):
        ml, m0, mr = _inputs(seed, b, n)
        rc, x, it, st = _noalloc(ml, m0, mr)
        assert rc == 0, (call, rc)
        xr, sr, ir = native.surfgf_batch(ml, m0, mr, itermax=50, errmax=1e-10)
        assert np.array_equal(st, sr) and np.array_equal(it, ir)
        err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
        assert err < TOL, (call, err)


def test_noalloc_padded_leading_dimension_on_a_caller_stream():
    """ld = n + 3 (padding as a Fortran array dimensioned larger than n, so
    every read and the in-place final inverse of x use the stride) on a
    non-default stream, against the allocating entry point and the oracle."""
    import torch
    s = torch.cuda.Stream()
    for call, (seed, b, n) in enumerate([(3, 3, 18), (10, 3, 29)]):
        ml, m0, mr = _inputs(seed, b, n)
        rc, x, it, st = _noalloc(ml, m0, mr, ld=n + 3, stream=s)
        assert rc == 0, (call, rc)
        assert np.isfinite(x).all()
        xr, sr, ir = native.surfgf_batch(ml, m0, mr, itermax=50, errmax=1e-10)
        assert np.array_equal(st, sr) and np.array_equal(it, ir)
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < TOL
        for q in range(b):
            xo, so, io = O.surfgfd(ml[q], m0[q], mr[q], itermax=50, errmax=1e-10)
            assert so == st[q] == 0 and io == it[q]
            assert np.linalg.norm(x[q] - xo) / np.linalg.norm(xo) < TOL, (call, q)


def test_noalloc_rejects_requests_over_its_limits():
    import torch
    n, b = 128, 64  # 64 * 8 * 128^2 * 16 B = 128 MiB > 32 MiB
    buf = torch.zeros((b, n, n), dtype=torch.complex128, device="cuda")  # in bounds for every input read
    p = buf.data_ptr()
    rc = _lib().skkr_gpu_surfgf_batch_noalloc(n, b, p, p, p, p, n, 50, 1e-8, None, None, None)
    assert rc == -6
    # more items than one grid dimension holds (the scratch would fit them at n = 1)
    small = torch.zeros(70000, dtype=torch.complex128, device="cuda")
    q = small.data_ptr()
    rc = _lib().skkr_gpu_surfgf_batch_noalloc(1, 65536, q, q, q, q, 1, 50, 1e-8, None, None, None)
    assert rc == -1
