"""The split-precision complex product restated on the host (CPU): digits
from the same slicing header the kernels include (tests/harness), the real
embedding [Re A, Im A] [[Re B, Im B], [-Im B, Re B]] over K' in groups of 16
complex indices [Re 16 | Im 16], slice pairs p + q <= S - 1 summed per level
in exact integers, levels weighted and scaled back.  Checks that the
embedding and the K' order give the complex product, that the error falls
with the slice count as the design says, and that the exact levels' sums stay
integers below 2^24 (what the FP32 tensor-core accumulators need)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("slp") / "libslp.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(ROOT, "tests", "harness", "slicing_host.cpp")], check=True)
    L = ctypes.CDLL(so)
    P, I = ctypes.c_void_p, ctypes.c_int
    L.slice_digits_eval.argtypes = [I, I, I, P, P, P]
    return L


def scale_exp(m):
    """log2 of the power-of-two scale of a max |x| (0 for zero)."""
    if m == 0:
        return 0
    return int(np.frexp(m)[1])


def digits(lib, x, es, S, DB):
    x = np.ascontiguousarray(x, float).ravel()
    e = np.ascontiguousarray(np.broadcast_to(es, x.shape), np.int32)
    out = np.zeros((x.size, S), np.int32)
    assert lib.slice_digits_eval(S, DB, x.size, x.ctypes.data, e.ctypes.data, out.ctypes.data) == 0
    return out


def kpos(k, im):
    return ((k >> 4) << 5) + (im << 4) + (k & 15)


def sliced_product(lib, A, B, S):
    """C = A B by the split-precision scheme, and the largest |level sum| of
    the exact levels (0..3)."""
    n, K = A.shape
    DB = 8 if K <= 128 else 7
    Se = 7 if (DB == 8 and S > 7) else S
    Kp = 32 * ((K + 15) // 16)
    # row scales of A, column scales of B over Re and Im together
    ea = np.array([scale_exp(np.abs(np.concatenate([A[i].real, A[i].imag])).max()) for i in range(n)])
    eb = np.array([scale_exp(np.abs(np.concatenate([B[:, j].real, B[:, j].imag])).max()) for j in range(n)])
    # A' (n x K') and B'^T (2n x K') digit planes, slice-major
    Ad = np.zeros((Se, n, Kp), np.int64)
    Bd = np.zeros((Se, 2 * n, Kp), np.int64)
    ks = np.arange(K)
    for i in range(n):
        dr = digits(lib, A[i].real, ea[i], Se, DB)  # (K, S)
        di = digits(lib, A[i].imag, ea[i], Se, DB)
        Ad[:, i, kpos(ks, 0)] = dr.T
        Ad[:, i, kpos(ks, 1)] = di.T
    for j in range(n):
        dr = digits(lib, B[:, j].real, eb[j], Se, DB)
        di = digits(lib, B[:, j].imag, eb[j], Se, DB)
        Bd[:, 2 * j, kpos(ks, 0)] = dr.T      # Re output column: [Re B, -Im B]
        Bd[:, 2 * j, kpos(ks, 1)] = -di.T
        Bd[:, 2 * j + 1, kpos(ks, 0)] = di.T  # Im output column: [Im B, Re B]
        Bd[:, 2 * j + 1, kpos(ks, 1)] = dr.T
    levels = np.zeros((Se, n, 2 * n), np.int64)
    for p in range(Se):
        for q in range(Se - p):
            levels[p + q] += Ad[p] @ Bd[q].T
    exact_max = int(np.abs(levels[:min(4, Se)]).max())
    # x = 2^es sum_p d_p 2^(-(DB-1) - DB p): a level l carries 2^(-2(DB-1) - DB l)
    acc = sum(levels[l].astype(float) * 2.0 ** (-2 * (DB - 1) - DB * l) for l in range(Se))
    acc = acc * np.ldexp(1.0, ea)[:, None] * np.repeat(np.ldexp(1.0, eb), 2)[None, :]
    return acc[:, 0::2] + 1j * acc[:, 1::2], exact_max


def crand(rng, *s):
    return rng.normal(size=s) + 1j * rng.normal(size=s)


@pytest.mark.parametrize("n,K", [(8, 16), (10, 37), (16, 128), (6, 150)])
def test_embedding_and_order_give_the_complex_product(lib, n, K):
    rng = np.random.default_rng(n + K)
    A, B = crand(rng, n, K), crand(rng, K, n)
    C, _ = sliced_product(lib, A, B, 7)
    ref = A @ B
    bound = (np.abs(A) @ np.abs(B)).max()
    assert np.abs(C - ref).max() < 1e-13 * bound


def test_error_falls_with_the_slice_count(lib):
    rng = np.random.default_rng(5)
    n, K = 12, 64
    A, B = crand(rng, n, K), crand(rng, K, n)
    ref = A @ B
    bound = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * K
    errs = []
    for S in (3, 4, 5, 6, 7):
        C, _ = sliced_product(lib, A, B, S)
        errs.append((np.abs(C - ref) / bound).max())
    # each slice adds 8 bits: the error shrinks by about 2^8 per slice (the
    # dropped pairs p + q > S - 1 dominate) until FP64 rounding takes over
    for e0, e1 in zip(errs[:-2], errs[1:-1]):
        assert e1 < e0 / 40
    assert errs[0] < 2.0 ** -20 and errs[2] < 2.0 ** -36 and errs[4] < 2.0 ** -50


@pytest.mark.parametrize("K,S", [(128, 7), (256, 7)])
def test_exact_levels_stay_below_2_24(lib, K, S):
    """Adversarial operands: every entry has the digits 127, 128, 128, 128,
    ... (8-bit digits, K' = 2K <= 256) or 63, 64, 64, 64, ... (7-bit, deeper
    products), and A = v (1 + i), B = v (1 - i) make every term of the real
    embedding add with the same sign.  The exact levels 0..3 (at most four
    slice pairs each) still stay below 2^24 in magnitude, so the tensor
    core's FP32 sums of them are exact integers; with 8-bit digits the bound
    is nearly reached."""
    DB = 8 if K <= 128 else 7
    h = 1 << (DB - 1)
    v = (h - 1 + sum(h / (2 * h) ** i for i in range(1, 4))) / h
    n = 4
    A = np.full((n, K), v * (1 + 1j))
    B = np.full((K, n), v * (1 - 1j))
    _, m = sliced_product(lib, A, B, S)
    assert m < 2 ** 24
    if DB == 8:
        assert m > 0.99 * 2 ** 24
