"""The C-ABI library loads and exports every entry point include/skkr_gpu.h
declares (CPU only: no compute call)."""
import ctypes
import os
import re

from skkr_budapest_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "skkr_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(skkr_gpu_\w+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    # compile a probe against the header and compare sizes/offsets with ctypes
    import subprocess
    src = tmp_path / "probe.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "skkr_gpu.h"\n'
        'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(skkr_sizes),'
        ' offsetof(skkr_sizes, errmax), offsetof(skkr_sizes, cpatol), offsetof(skkr_sizes, slices),'
        ' sizeof(skkr_rtable), offsetof(skkr_rtable, blkmap), sizeof(skkr_status),'
        ' offsetof(skkr_status, max_refine_resid)); return 0;}\n')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    S, R, T = native.Sizes, native.RTable, native.Status
    want = [ctypes.sizeof(S), S.errmax.offset, S.cpatol.offset, S.slices.offset, ctypes.sizeof(R),
            R.blkmap.offset, ctypes.sizeof(T), T.max_refine_resid.offset]
    assert got == want


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    monkeypatch.setattr(native, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(native, "_lib", None)
    import pytest
    with pytest.raises(RuntimeError):
        native.lib()


def test_argument_checks_before_any_device_call():
    # invalid arguments are refused with SKKR_ERR_ARG before CUDA is touched,
    # so these run without a GPU
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    ARG = -1
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.skkr_gpu_tauij.argtypes = [P, I, P, P, P, P, P, P, P, I, P]
    assert lib.skkr_gpu_tauij(None, 1, None, None, None, None, None, None, None, 32, None) == ARG
    import numpy as np
    buf = np.zeros(2 * 64 * 64)
    al = np.zeros(16)
    bp = buf.ctypes.data
    lib.skkr_gpu_phystau2.argtypes = [I, I, P, P, P, P, P, I]
    assert lib.skkr_gpu_phystau2(1, 3, bp, bp, al.ctypes.data, None, al.ctypes.data, 32) == ARG
    assert lib.skkr_gpu_phystau2(5, 3, bp, bp, al.ctypes.data, bp, al.ctypes.data, 32) == ARG    # mode
    assert lib.skkr_gpu_phystau2(1, 4, bp, bp, al.ctypes.data, bp, al.ctypes.data, 64) == ARG    # lmax
    assert lib.skkr_gpu_phystau2(1, 3, bp, bp, al.ctypes.data, bp, al.ctypes.data, 31) == ARG    # ld < 32
    lib.skkr_gpu_set_mixed_policy.argtypes = [P, D, D, I, D]
    assert lib.skkr_gpu_set_mixed_policy(None, 1e-3, 0.0, 0, 1e-2) == ARG
    s = native.Sizes()
    s.mode, s.lmax, s.nprc, s.ngeff = 7, 3, 3, 1
    out = ctypes.c_void_p()
    lib.skkr_gpu_create.argtypes = [P, P]
    assert lib.skkr_gpu_create(ctypes.cast(ctypes.pointer(s), P), ctypes.cast(ctypes.pointer(out), P)) == ARG
    s.mode, s.precision = 1, 5          # unknown precision
    assert lib.skkr_gpu_create(ctypes.cast(ctypes.pointer(s), P), ctypes.cast(ctypes.pointer(out), P)) == ARG


def test_size_limits_at_creation():
    # the checks of skkr_gpu_create that run before any CUDA call: principal
    # layers above the 256-row kernels, non-uniform principal layers, slice
    # counts outside 3..8, more than 8 group elements, no interface PL
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    P = ctypes.c_void_p
    lib.skkr_gpu_create.argtypes = [P, P]
    ARG, UNSUPPORTED = -1, -5

    def create(mode=1, lmax=3, nprc=3, pl=4, ngeff=8, slices=0, ninprc=None):
        s = native.Sizes()
        s.mode, s.lmax, s.nprc, s.ngeff, s.precision, s.slices = mode, lmax, nprc, ngeff, 0, slices
        for i, v in enumerate(ninprc or [pl] * (nprc + 2)):
            s.ninprc[i] = v
        out = ctypes.c_void_p()
        return lib.skkr_gpu_create(ctypes.cast(ctypes.pointer(s), P), ctypes.cast(ctypes.pointer(out), P))

    assert create(mode=2, lmax=3, pl=5) == UNSUPPORTED        # BdG lmax 3: 5 x 64 = 320 rows
    assert create(mode=1, lmax=3, pl=9) == UNSUPPORTED        # relativistic: 9 x 32 = 288 rows
    assert create(ninprc=[4, 4, 2, 4, 4]) == UNSUPPORTED      # non-uniform principal layers
    assert create(slices=2) == ARG
    assert create(slices=9) == ARG
    assert create(ngeff=9) == ARG
    assert create(nprc=0, ninprc=[4, 4]) == ARG
    assert create(nprc=17, ninprc=[4] * 18) == ARG


def test_mlp_argument_checks_before_any_device_call():
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    ARG = -1
    lib.skkr_gpu_mlp_forward.argtypes = [I, P, P, I, P, P]
    lib.skkr_gpu_mlp_grad.argtypes = [I, P, P, I, P, P, P, P, P]
    lib.skkr_gpu_mlp_train.argtypes = [I, P, P, I, P, P, P, I, D, D, I, P, P, P]
    dims = np.array([3, 4, 2], np.int32)
    bad = np.array([3, 0, 2], np.int32)
    big = np.array([3, 5000, 2], np.int32)
    buf = np.zeros(64)
    d, b, g = dims.ctypes.data, buf.ctypes.data, bad.ctypes.data
    assert lib.skkr_gpu_mlp_forward(0, d, b, 4, b, b) == ARG          # no layer
    assert lib.skkr_gpu_mlp_forward(9, d, b, 4, b, b) == ARG          # more than 8
    assert lib.skkr_gpu_mlp_forward(2, g, b, 4, b, b) == ARG          # a zero width
    assert lib.skkr_gpu_mlp_forward(2, big.ctypes.data, b, 4, b, b) == ARG
    assert lib.skkr_gpu_mlp_forward(2, d, b, 0, b, b) == ARG          # no row
    assert lib.skkr_gpu_mlp_forward(2, d, None, 4, b, b) == ARG
    held = np.zeros(4, np.uint8)                                      # every row held out
    assert lib.skkr_gpu_mlp_grad(2, d, b, 4, b, b, held.ctypes.data, b, b) == ARG
    assert lib.skkr_gpu_mlp_train(2, d, b, 4, b, b, None, 0, 1e-3, 0.0, 20, b, b, b) == ARG   # no epoch
    assert lib.skkr_gpu_mlp_train(2, d, b, 4, b, b, None, 5, 0.0, 0.0, 20, b, b, b) == ARG   # lr 0
    assert lib.skkr_gpu_mlp_train(2, d, b, 4, b, b, None, 5, 1e-3, -1.0, 20, b, b, b) == ARG  # wd < 0


def test_kambe_argument_checks_before_any_device_call():
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.skkr_gpu_kambe_dlm.argtypes = [I, D, D, P, P, I, P, I, P, I, D, D, D, D, P]
    b = np.zeros(64).ctypes.data
    ok = (0.5, 0.01, b, b, 4, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, b)
    assert lib.skkr_gpu_kambe_dlm(0, *ok) == -1                                     # no item
    assert lib.skkr_gpu_kambe_dlm(1, 0.5, 0.01, b, b, 7, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, b) == -1   # lmax2
    assert lib.skkr_gpu_kambe_dlm(1, 0.5, 0.01, b, b, 4, b, 3, b, 3, 0.0, 1.0, 12.0, 40.0, b) == -1    # area
    assert lib.skkr_gpu_kambe_dlm(1, 0.0, 0.0, b, b, 4, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, b) == -1    # E = 0
    assert lib.skkr_gpu_kambe_dlm(1, 0.5, 0.01, None, b, 4, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, b) == -1


def test_kambe_blocks_argument_checks_before_any_device_call():
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.skkr_gpu_kambe_alm.argtypes = [I, D, D, P, P, I, P, I, P, I, D, D, D, D, P]
    b = np.zeros(64).ctypes.data
    assert lib.skkr_gpu_kambe_alm(1, 0.5, 0.01, b, b, 4, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, b) == -1   # lmax 4
    assert lib.skkr_gpu_kambe_alm(0, 0.5, 0.01, b, b, 2, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, b) == -1   # no item
    assert lib.skkr_gpu_kambe_alm(1, 0.5, 0.01, b, b, 2, b, 0, b, 3, 23.1, 1.0, 12.0, 40.0, b) == -1   # no g


def test_kambe_screened_argument_checks_before_any_device_call():
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    lib = ctypes.CDLL(native.LIB_PATH)
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.skkr_gpu_kambe_screened.argtypes = [I, D, D, P, I, P, P, I, P, I, P, I, D, D, D, D, I, I, P]
    b = np.zeros(256).ctypes.data
    # 33 layers of lmax 3 exceed the 512-row inverse; the centre must leave jmax layers on each side
    assert lib.skkr_gpu_kambe_screened(1, 0.5, 0.01, b, 33, b, b, 3, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, 8, 2, b) == -1
    assert lib.skkr_gpu_kambe_screened(1, 0.5, 0.01, b, 8, b, b, 2, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, 1, 2, b) == -1
    assert lib.skkr_gpu_kambe_screened(1, 0.5, 0.01, b, 8, b, b, 2, b, 3, b, 3, 23.1, 1.0, 12.0, 40.0, 6, 2, b) == -1
