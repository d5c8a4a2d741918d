"""The Faddeeva function of skkr_budapest_gb300/csrc/faddeeva.cuh (Weideman's
rational approximation, the erfc of the Kambe sums) compiled for the host
from the same header, against scipy.special.wofz over the complex plane
(CPU).  Also: its coefficient table is the published construction."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest
from scipy.special import wofz

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "skkr_budapest_gb300", "csrc", "faddeeva.cuh")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("fad") / "libfad.so")
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-o", so, os.path.join(ROOT, "tests", "harness",
                                                                            "faddeeva_host.cpp")], check=True)
    L = ctypes.CDLL(so)
    P = ctypes.c_void_p
    L.faddeeva_eval.argtypes = [ctypes.c_int, P, P, P, P]
    return L


def _w(lib, z):
    z = np.ascontiguousarray(z, complex)
    zr, zi = np.ascontiguousarray(z.real), np.ascontiguousarray(z.imag)
    wr, wi = np.zeros(len(z)), np.zeros(len(z))
    lib.faddeeva_eval(len(z), zr.ctypes.data, zi.ctypes.data, wr.ctypes.data, wi.ctypes.data)
    return wr + 1j * wi


def test_upper_half_plane(lib):
    rng = np.random.default_rng(0)
    z = np.concatenate([r * np.exp(1j * rng.uniform(0, np.pi, 500)) for r in (0.01, 0.3, 1, 3, 6, 10, 30, 100)])
    z = np.concatenate([z, rng.uniform(-20, 20, 500) + 0j, 1j * rng.uniform(0, 50, 100), [0j]])
    ref = wofz(z)
    assert np.max(np.abs(_w(lib, z) - ref) / np.abs(ref)) < 2e-14


def test_lower_half_plane(lib):
    # w(z) = 2 exp(-z^2) - w(-z): relative accuracy where exp(-z^2) stays finite
    rng = np.random.default_rng(1)
    z = np.concatenate([r * np.exp(-1j * rng.uniform(0, np.pi, 500)) for r in (0.01, 0.3, 1, 3, 6)])
    ref = wofz(z)
    assert np.max(np.abs(_w(lib, z) - ref) / np.abs(ref)) < 1e-12


def test_arguments_of_the_kambe_sums(lib):
    # the arguments incgamma / ilkam / delkam pass to cerf for the contour
    # energies of the workloads (kamstr.f: alpha = E A / 4 pi, i sqrt(x), +-sqrt(x) + i a)
    import kambe as K
    calls = []
    orig = K.cerf
    K.cerf = lambda z: (calls.append(complex(z)), orig(z))[1]
    try:
        lat = K.Lattice2D([4.808326, 0.0], [0.0, 4.808326])
        for e in (-0.45 + 0.06j, 0.3 + 0.01j, 0.7 + 1e-4j):
            for sep in ((0.0, 0.0, 0.0), (1.2, 0.7, 3.4), (2.404, 2.404, 0.0)):
                K.kambe_dlm(e, 0.21, 0.07, sep, 4, lat)
    finally:
        K.cerf = orig
    z = np.array(calls)
    z = z[np.isfinite(wofz(z)) & (np.abs(wofz(z)) < 1e300)]
    ref = wofz(z)
    err = np.abs(_w(lib, z) - ref) / np.maximum(np.abs(ref), 1e-300)
    assert len(z) > 1000 and np.max(err) < 1e-12


def test_coefficients_are_the_published_construction():
    n = 40
    m = 2 * n
    k = np.arange(-m + 1, m)
    L = np.sqrt(n / np.sqrt(2))
    t = L * np.tan(k * np.pi / m / 2)
    f = np.concatenate([[0.0], np.exp(-t ** 2) * (L ** 2 + t ** 2)])
    a = (np.real(np.fft.fft(np.fft.fftshift(f))) / (2 * m))[1:n + 1][::-1]
    src = open(HDR).read()
    body = src[src.index("const double a[SKKR_WEIDEMAN_N] = {"):]
    body = body[body.index("{") + 1:body.index("};")]
    tab = np.array([float(v) for v in re.findall(r"[-+]?\d\.\d+e[-+]\d+", body)])
    assert len(tab) == n and np.allclose(tab, a, rtol=0, atol=1e-30 + 1e-15 * np.abs(a).max())
    assert abs(float(re.search(r"SKKR_WEIDEMAN_L ([0-9.e+-]+)", src).group(1)) - L) < 1e-15
