"""The oracle's generators against the reference's own sample run
(sample/02-layer-scf: contour energies, k-mesh sizes and the 2D lattice cell
printed in its log)."""
import json
import os

import numpy as np

import oracle as O
from skkr_budapest_gb300 import synth as S

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sample02_contour.json")))


def test_zmesh_energies_match_sample_log():
    z, w = O.zmesh_semicircle(G["nepanel"], G["ebottom"], G["etop"], G["eps"])
    ref = np.array([complex(a, b) for a, b in G["energies"]])
    # the log prints 8 decimals
    assert np.max(np.abs(z.real - ref.real)) < 6e-9
    assert np.max(np.abs(z.imag - ref.imag)) < 6e-9


def test_package_zmesh_equals_oracle():
    z0, w0 = O.zmesh_semicircle(G["nepanel"], G["ebottom"], G["etop"], G["eps"])
    z1, w1 = S.zmesh_semicircle(G["nepanel"], G["ebottom"], G["etop"], G["eps"])
    assert np.max(np.abs(z0 - z1)) < 1e-14
    assert np.max(np.abs(w0 - w1)) < 1e-14


def test_kmesh_sizes_match_sample_log():
    # kset per energy from KSETTAB/INTAB (rsp-scf/readini.f:401-409)
    ksets = [k for k, cnt in G["ksettab"] for _ in range(cnt)]
    for kset, nk_ref in zip(ksets, G["nk"]):
        xk, wk = O.kmesh2d_ibz(kset, G["i2dlat"], "C2v", G["a2d"], G["beta"], G["delta"])
        assert len(xk) == nk_ref
        assert abs(wk.sum() - 1.0) < 1e-12


def test_legzero_is_gauss_legendre():
    for n in (3, 8, 16, 24):
        x, w = O.legzero(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        assert np.allclose(x, xr, atol=1e-13) and np.allclose(w, wr, atol=1e-13)


def test_package_square_kmesh_equals_oracle():
    for n in (5, 22):
        xo, wo = O.kmesh2d_ibz(n, 4, "C4v", 4.8)
        xs, ws = S.kmesh_square_c4v(n, 4.8)
        assert np.allclose(xo, xs, atol=1e-14) and np.allclose(wo, ws, atol=1e-14)


def test_alpha_package_equals_oracle():
    for e in (0.3 + 0.2j, -0.4 + 0.01j, 0.69 + 0.005j):
        a0 = O.alpha_sqwell(e, 2.0, 3.2, 3)
        a1 = S.alpha_sqwell(e, 2.0, 3.2, 3)
        assert np.allclose(a0, a1, rtol=1e-12, atol=1e-14)


def test_kambe_lattice_matches_sample_log():
    # routine VECTOR2D of the sample run prints the 2D cell of the bcc(110)
    # slab (centered rectangular, i2dlat = 2): a2 = (a/2, beta a/2), the
    # unit-cell area and the reciprocal cell the Kambe sums run over (10
    # decimals in the log)
    import kambe as K
    a1, a2 = (np.array(v) for v in G["a_vectors"])
    assert np.allclose(a2, [a1[0] / 2, G["beta"] * a1[0] / 2], atol=1e-9)
    lat = K.Lattice2D(a1, a2)
    assert abs(lat.area - G["area2d"]) < 1e-7
    b1, b2 = (np.array(v) for v in G["b_vectors"])
    assert np.allclose(lat.b1, b1, atol=1e-9) and np.allclose(lat.b2, b2, atol=1e-9)
