"""The Kambe lattice sums written for the device
(skkr_budapest_gb300/csrc/kambe_dev.cuh), compiled for the host from the
same header, against the oracle's restatement of main/kamstr.f
(oracle/kambe.py) on the same lattice vectors (CPU)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import kambe as K

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
A2D = 4.808326112068523
LAT = K.Lattice2D([A2D, 0.0], [0.0, A2D])
GCUT, RCUT = 12.0, 40.0


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("kam") / "libkam.so")
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-o", so,
                    os.path.join(ROOT, "tests", "harness", "kambe_host.cpp")], check=True)
    L = ctypes.CDLL(so)
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.kambe_eval.argtypes = [D, D, D, D, D, D, D, I, P, I, P, I, D, D, D, D, P]
    return L


def _dev(lib, e, k, sep, lmax2):
    g = np.ascontiguousarray(LAT.gvecs(GCUT + 2.0))
    r = np.ascontiguousarray(LAT.rvecs(RCUT + 15.0))
    out = np.zeros(2 * (lmax2 + 1) ** 2)
    lib.kambe_eval(e.real, e.imag, k[0], k[1], *sep, lmax2, g.ctypes.data, len(g), r.ctypes.data, len(r),
                   LAT.area, 1.0, GCUT, RCUT, out.ctypes.data)
    return out[0::2] + 1j * out[1::2]


@pytest.mark.parametrize("e", [0.3 + 0.01j, 0.4 + 0.6j, -0.45 + 0.06j, 0.7 + 1e-4j])
@pytest.mark.parametrize("sep", [(0.0, 0.0, 0.0), (1.2, 0.7, 3.4), (0.5 * A2D, 0.5 * A2D, 0.0), (0.4, -1.1, -6.8)])
@pytest.mark.parametrize("lmax2", [4, 6])
def test_device_form_equals_the_oracle(lib, e, sep, lmax2):
    k = (0.21, 0.07)
    d = _dev(lib, e, k, sep, lmax2)
    ref = K.kambe_dlm(e, *k, sep, lmax2, LAT, gcut=GCUT, rcut=RCUT)
    # in plane kamstr shifts the pair to s_z = 1.1e-4, and delkam's upward
    # recursion multiplies by (2 / (k_z s_z))^2 per step: at lmax2 = 6 the two
    # builds' rounding then differs by up to 1.5e-10, while both sit 8e-5
    # from the unshifted lattice sum (the method's own error there)
    in_plane = sep[2] == 0.0 and any(sep[:2])
    assert np.abs(d - ref).max() < (1e-9 if in_plane else 1e-12) * np.abs(ref).max()


@pytest.mark.parametrize("e", [0.3 + 0.01j, 0.4 + 0.6j])
@pytest.mark.parametrize("sep", [(0.0, 0.0, 0.0), (1.2, 0.7, 3.4), (0.4, -1.1, -6.8)])
@pytest.mark.parametrize("lmax", [2, 3])
def test_device_blocks_equal_kamstr(lib, e, sep, lmax):
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.kambe_alm_eval.argtypes = [D, D, D, D, D, D, D, I, P, I, P, I, D, D, D, P, P]
    g = np.ascontiguousarray(LAT.gvecs(GCUT + 2.0))
    r = np.ascontiguousarray(LAT.rvecs(RCUT + 15.0))
    coef = np.ascontiguousarray(K.alm_coef(lmax).view(np.float64))
    lm = (lmax + 1) ** 2
    out = np.zeros(2 * lm * lm)
    k = (0.21, 0.07)
    lib.kambe_alm_eval(e.real, e.imag, *k, *sep, lmax, g.ctypes.data, len(g), r.ctypes.data, len(r), LAT.area,
                       GCUT, RCUT, coef.ctypes.data, out.ctypes.data)
    got = (out[0::2] + 1j * out[1::2]).reshape(lm, lm)
    ref = K.kamstr(e, *k, lmax, sep, LAT, gcut=GCUT, rcut=RCUT)
    assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("lmax", [0, 1, 2, 3])
def test_library_coefficient_table_equals_the_oracle(lmax):
    # skkr_gpu_kambe_coef is host code (no device call), so it runs here
    from skkr_budapest_gb300 import native
    L = ctypes.CDLL(native.LIB_PATH)
    L.skkr_gpu_kambe_coef.argtypes = [ctypes.c_int, ctypes.c_void_p]
    lm, lm2 = (lmax + 1) ** 2, (2 * lmax + 1) ** 2
    out = np.zeros(2 * lm * lm * lm2)
    assert L.skkr_gpu_kambe_coef(lmax, out.ctypes.data) == 0
    got = (out[0::2] + 1j * out[1::2]).reshape(lm, lm, lm2)
    assert np.abs(got - K.alm_coef(lmax)).max() < 1e-13
    assert L.skkr_gpu_kambe_coef(4, out.ctypes.data) == -1


def test_slab_chain_of_the_device_entry_point(lib):
    # the element functions of k_slab_assemble / k_slab_extract (the same
    # header) with the host-built blocks; numpy stands in for the batched
    # Gauss-Jordan and GEMM the entry point runs between them
    from skkr_budapest_gb300 import native
    from skkr_budapest_gb300 import synth as S
    from skkr_budapest_gb300 import workloads as W
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.kambe_alm_eval.argtypes = [D, D, D, D, D, D, D, I, P, I, P, I, D, D, D, P, P]
    lib.slab_assemble_eval.argtypes = [I, I, I, P, P, I, P, P, P, I, P, P]
    lib.slab_extract_eval.argtypes = [I, I, I, I, I, P, P]
    lib.slab_cache_eval.argtypes = [I, I, I, I, I, P, I, P, P]
    spec = W.plain_fcc(nset=4)
    st = spec.stacking
    lat = K.Lattice2D([st.a2d, 0.0], [0.0, st.a2d])
    _, _, dnn = S.cluster(st, 1)
    ce = complex(spec.energies[8])
    lmax = spec.lmax
    al = S.alpha_sqwell(ce, 4.0, 0.5 * dnn, lmax)
    nl, centre, jmax = 6, 3, 2
    lm, lm2 = (lmax + 1) ** 2, (2 * lmax + 1) ** 2
    pos = np.ascontiguousarray([st.site(n, 0, 0) for n in range(nl)], np.float64)
    kpts = np.ascontiguousarray([(0.31, 0.12), (0.5, 0.2)], np.float64)
    Lb = ctypes.CDLL(native.LIB_PATH)
    Lb.skkr_gpu_kambe_coef.argtypes = [I, P]
    coef = np.zeros(2 * lm * lm * lm2)
    Lb.skkr_gpu_kambe_coef(lmax, coef.ctypes.data)
    g = np.ascontiguousarray(lat.gvecs(14.0))
    r = np.ascontiguousarray(lat.rvecs(55.0))
    # the lattice sums once per distinct separation, the pairs through a map
    # (this stacking's sites alternate by half a lattice vector: 15
    # separations for 6 layers instead of 36 pairs)
    seps, pmap = [], np.zeros((nl, nl), np.int32)
    for a in range(nl):
        for b in range(nl):
            sv = tuple(np.round(pos[a] - pos[b], 9))
            if sv not in seps:
                seps.append(sv)
            pmap[a, b] = seps.index(sv)
    assert len(seps) == 15
    alm = np.zeros((len(kpts), len(seps), lm, lm), complex)
    for ik, k in enumerate(kpts):
        for q, sv in enumerate(seps):
            out = np.zeros(2 * lm * lm)
            lib.kambe_alm_eval(ce.real, ce.imag, k[0], k[1], *sv, lmax, g.ctypes.data, len(g), r.ctypes.data,
                               len(r), lat.area, 12.0, 40.0, coef.ctypes.data, out.ctypes.data)
            alm[ik, q] = (out[0::2] + 1j * out[1::2]).reshape(lm, lm)
    alm = np.ascontiguousarray(alm)
    alpha = np.ascontiguousarray(np.array([al] * nl, complex))
    N = nl * lm
    G = np.zeros((len(kpts), N, N), complex)
    A = np.zeros_like(G)
    lib.slab_assemble_eval(len(kpts), nl, lm, alm.ctypes.data, np.ascontiguousarray(pmap).ctypes.data, len(seps),
                           kpts.ctypes.data, pos.ctypes.data, alpha.ctypes.data, lmax + 1, G.ctypes.data,
                           A.ctypes.data)
    # the buffers are column-major per k: transpose to (row, col)
    G, A = G.transpose(0, 2, 1), A.transpose(0, 2, 1)
    X = np.ascontiguousarray(np.array([Gk @ np.linalg.inv(Ak) for Gk, Ak in zip(G, A)]).transpose(0, 2, 1))
    out = np.zeros((len(kpts), 2 * jmax + 1, lm, lm), complex)
    lib.slab_extract_eval(len(kpts), nl, lm, centre, jmax, X.ctypes.data, out.ctypes.data)
    # the same blocks written into a structure-constant cache of 7 blocks per
    # k (column-major), offset j at block blk[j], offset +2 left out
    blk = np.array([4, 0, 6, 2, -1], np.int32)
    cache = np.zeros((len(kpts), 7, lm, lm), complex)
    lib.slab_cache_eval(len(kpts), nl, lm, centre, jmax, blk.ctypes.data, 7, X.ctypes.data, cache.ctypes.data)
    for ik in range(len(kpts)):
        for j in range(2 * jmax + 1):
            if blk[j] >= 0:
                assert np.array_equal(cache[ik, blk[j]].T, out[ik, j])
        assert not cache[ik, [1, 3, 5]].any()
    for ik, k in enumerate(kpts):
        gs = K.screened_slab(ce, k[0], k[1], lmax, pos, [al] * nl, lat)
        ref = np.array([gs[centre, centre + j] for j in range(-jmax, jmax + 1)])
        assert np.abs(out[ik] - ref).max() < 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("e", [0.4 + 0.6j, 0.3 + 0.01j, -0.45 + 0.06j, 0.7 + 1e-4j])
@pytest.mark.parametrize("sep", [(0.5 * A2D, 0.5 * A2D, 6.8), (0.3, -0.8, 10.2), (0.0, 0.0, -13.6),
                                 (0.5 * A2D, 0.5 * A2D, -6.8)])
@pytest.mark.parametrize("lmax", [2, 3])
def test_device_plane_wave_form_equals_directg(lib, e, sep, lmax):
    """The plane-wave form of the device (directg_alm, the terms of its
    kernel) against the oracle's directg: gp for s_z > 0, gm of -s for
    s_z < 0, on the g vectors within 14 a.u.^-1 of the origin (the oracle
    takes |k + g| <= 30; the rest is below e^{-14 |s_z|})."""
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.directg_eval.argtypes = [D, D, D, D, D, D, D, I, P, I, D, P]
    g = np.ascontiguousarray(LAT.gvecs(14.0))
    lm = (lmax + 1) ** 2
    out = np.zeros(2 * lm * lm)
    k = (0.21, 0.07)
    lib.directg_eval(e.real, e.imag, *k, *sep, lmax, g.ctypes.data, len(g), LAT.area, out.ctypes.data)
    got = (out[0::2] + 1j * out[1::2]).reshape(lm, lm)
    s = np.asarray(sep)
    ref = K.directg(e, *k, lmax, s, LAT)[0] if s[2] > 0 else K.directg(e, *k, lmax, -s, LAT)[1]
    assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()
    # and gstore's choice for this pair is the plane-wave form
    assert abs(s[2]) * LAT.bmin >= 5.0
    assert np.abs(got - K.gstore_block(e, *k, lmax, s, LAT)).max() < 1e-12 * np.abs(ref).max()
