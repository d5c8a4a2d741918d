"""The aliasing test that decides whether a split-precision product may read
its B operand while it writes C, D and E (csrc/common.cuh mref_overlap),
compiled for the host, against a brute-force element-set intersection
(CPU).  A wrong "apart" would let CTAs read elements others already wrote."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("ovl") / "libovl.so")
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-I/usr/local/cuda/include", "-o", so,
                    os.path.join(ROOT, "tests", "harness", "overlap_host.cpp")], check=True)
    L = ctypes.CDLL(so)
    ll, i = ctypes.c_longlong, ctypes.c_int
    L.overlap_eval.argtypes = [ll, ll, ll, i, ll, ll, ll, i, ctypes.c_void_p, i, i, i]
    return L


def _elems(off, sk, sc, ld, mp, nk, nc, n):
    s = set()
    for k in range(nk):
        for c in range(nc):
            b = off + k * sk + mp[c] * sc
            for j in range(n):
                s.update(range(b + j * ld, b + j * ld + n))
    return s


def _case(lib, a, b, mp, nk, nc, n):
    m = np.ascontiguousarray(mp, np.int32)
    got = lib.overlap_eval(*a, *b, m.ctypes.data, nk, nc, n)
    true = bool(_elems(*a, mp, nk, nc, n) & _elems(*b, mp, nk, nc, n))
    return got, true


def test_interleaved_buffers_are_apart(lib):
    # nbuf n x n buffers per item, items nbuf n^2 apart (the tau2d work layout)
    n, nbuf, nc, nk = 4, 5, 2, 3
    MB = n * n
    mp = list(range(nc))
    sk, sc = nc * nbuf * MB, nbuf * MB
    for b1 in range(nbuf):
        for b2 in range(nbuf):
            got, true = _case(lib, (b1 * MB, sk, sc, n), (b2 * MB, sk, sc, n), mp, nk, nc, n)
            assert got == (b1 == b2) and true == (b1 == b2)


def test_never_apart_when_sharing(lib):
    rng = np.random.default_rng(3)
    for _ in range(400):
        n = int(rng.integers(1, 5))
        ld = n + int(rng.integers(0, 3))
        nk, nc = int(rng.integers(1, 4)), int(rng.integers(1, 4))
        mp = [int(x) for x in rng.permutation(4)[:nc]]
        sk = int(rng.integers(0, 3)) * n * ld * int(rng.integers(1, 5))
        sc = n * ld * int(rng.integers(0, 4))
        if rng.random() < 0.5:
            skb, scb = sk, sc
        else:
            skb, scb = int(rng.integers(0, 60)), int(rng.integers(0, 30))
        a = (int(rng.integers(0, 40)), sk, sc, ld)
        b = (int(rng.integers(0, 40)), skb, scb, ld)
        got, true = _case(lib, a, b, mp, nk, nc, n)
        if true:
            assert got == 1, (a, b, mp, nk, nc, n)
