"""The BF16 digit slicing of the split-precision products
(skkr_budapest_gb300/csrc/slicing.cuh), compiled for the host from the same
header the kernels include, against exact integer arithmetic (CPU):
fixed-point rounding, the balanced digits (and the carry-chain form they
replaced, digit for digit), and the BF16 words the tiles receive."""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = [(3, 8), (4, 8), (5, 8), (6, 8), (7, 8), (3, 7), (5, 7), (7, 7), (8, 7)]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("slc") / "libslc.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(ROOT, "tests", "harness", "slicing_host.cpp")], check=True)
    L = ctypes.CDLL(so)
    P, I = ctypes.c_void_p, ctypes.c_int
    L.slice_digits_eval.argtypes = [I, I, I, P, P, P]
    L.slice4_eval.argtypes = [I, I, P, P, I, I, P, P]
    L.fix_round_eval.argtypes = [ctypes.c_double, I]
    L.fix_round_eval.restype = ctypes.c_longlong
    return L


def exact_round(x, E):
    """round(x 2^E), halves away from zero, in exact integer arithmetic."""
    num, den = float(x).as_integer_ratio()
    if E >= 0:
        num <<= E
    else:
        den <<= -E
    q, r = divmod(abs(num), den)
    if 2 * r >= den:
        q += 1
    return -q if num < 0 else q


def carry_digits(Y, S, DB):
    """Balanced digits by the carry chain (least significant first: a digit
    above 2^(DB-1) borrows 2^DB from the next), most significant first."""
    u, half, out, carry = abs(Y), 1 << (DB - 1), [], 0
    for q in range(S):
        d = ((u >> (DB * q)) & ((1 << DB) - 1)) + carry
        carry = int(d > half)
        d -= carry << DB
        out.append(-d if Y < 0 else d)
    return out[::-1]


def samples(rng, n):
    es = rng.integers(-30, 30, n)
    frac = rng.uniform(0.5, 1.0, n) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    drop = np.where(rng.random(n) < 0.8, 0, rng.integers(0, 70, n))
    x = np.ldexp(frac, es - drop)
    # the largest values below sigma (their rounding reaches the top digit's
    # largest value), exact powers of two, zeros
    k = n // 10
    x[:k] = np.ldexp(np.where(rng.random(k) < 0.5, -1.0, 1.0) * (1 - 2.0 ** -53), es[:k])
    x[k:2 * k] = np.ldexp(0.5, es[k:2 * k] - rng.integers(0, 40, k))
    x[2 * k:2 * k + 5] = 0.0
    return x, es.astype(np.int32)


def test_fix_round_is_exact(lib):
    rng = np.random.default_rng(1)
    x, es = samples(rng, 3000)
    for v, e in zip(x, es):
        E = 55 - int(e)
        assert lib.fix_round_eval(float(v), E) == exact_round(v, E)


@pytest.mark.parametrize("S,DB", CASES)
def test_digits_are_the_balanced_digits(lib, S, DB):
    rng = np.random.default_rng(S * 10 + DB)
    x, es = samples(rng, 4000)
    out = np.zeros((len(x), S), np.int32)
    assert lib.slice_digits_eval(S, DB, len(x), x.ctypes.data, es.ctypes.data, out.ctypes.data) == 0
    half = 1 << (DB - 1)
    top_seen = False
    for v, e, d in zip(x, es, out):
        Y = exact_round(v, (DB - 1) + DB * (S - 1) - int(e))
        assert sum(int(c) << (DB * (S - 1 - q)) for q, c in enumerate(d)) == Y
        assert list(d) == carry_digits(Y, S, DB)
        lo = d[1:] * (1 if Y >= 0 else -1)
        assert np.all(lo >= -(half - 1)) and np.all(lo <= half)
        assert abs(int(d[0])) <= half
        top_seen |= abs(int(d[0])) == half
    assert top_seen


@pytest.mark.parametrize("S,DB", CASES)
@pytest.mark.parametrize("wshift", [0, 16])
def test_words_hold_the_scaled_digits_as_bf16(lib, S, DB, wshift):
    rng = np.random.default_rng(7 + S + DB + wshift)
    for _ in range(200):
        es = int(rng.integers(-10, 10))
        re = np.ldexp(rng.uniform(-1, 1, 4), es)
        im = np.ldexp(rng.uniform(-1, 1, 4), es)
        if rng.random() < 0.2:
            re[int(rng.integers(0, 4))] = 0.0
        wr = np.zeros(2 * S, np.uint32)
        wi = np.zeros(2 * S, np.uint32)
        assert lib.slice4_eval(S, DB, re.ctypes.data, im.ctypes.data, es, wshift, wr.ctypes.data,
                               wi.ctypes.data) == 0
        for part, w in ((re, wr), (im, wi)):
            dg = np.zeros((4, S), np.int32)
            esv = np.full(4, es, np.int32)
            lib.slice_digits_eval(S, DB, 4, np.ascontiguousarray(part).ctypes.data, esv.ctypes.data,
                                  dg.ctypes.data)
            for e in range(4):
                for p in range(S):
                    word = int(w[2 * p + e // 2])
                    half16 = (word >> (16 * (e % 2))) & 0xFFFF
                    val = np.array([half16 << 16], np.uint32).view(np.float32)[0]
                    assert float(val) == math.ldexp(int(dg[e, p]), wshift - DB * p)
