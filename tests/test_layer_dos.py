"""Layer DOS inputs and the oracle's DOS (nrsp-scf/moment.f:47-110 with
locquant.f:86-126; rsp-scf/moment.f:60-140 with locquant.f:197-232) on CPU."""
import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W

sp = pytest.importorskip("scipy.special")


def _fg_quadrature(p2, v, radius, l, nq=400):
    """F, G by Gauss-Legendre quadrature of the matched radial solutions."""
    ck, q = S.kappa_of(p2), S.kappa_of(complex(p2) - v)
    tand = S._tan_delta(ck, q, radius, l)[l]
    react = -tand / ck
    t = react / (1 + 1j * ck * react)
    x, w = np.polynomial.legendre.leggauss(nq)
    r, w = (x + 1) * radius / 2, w * radius / 2
    jk = sp.spherical_jn(l, ck * radius)
    hk = jk + 1j * sp.spherical_yn(l, ck * radius)
    a = (jk / t - 1j * ck * hk) / sp.spherical_jn(l, q * radius)
    f, df = sp.spherical_jn(l, q * radius), q * sp.spherical_jn(l, q * radius, derivative=True)
    g, dg = sp.spherical_yn(l, q * radius), q * sp.spherical_yn(l, q * radius, derivative=True)
    j0, dj0 = jk, ck * sp.spherical_jn(l, ck * radius, derivative=True)
    det = f * dg - df * g
    b, c = (j0 * dg - dj0 * g) / det, (f * dj0 - df * j0) / det
    z = a * sp.spherical_jn(l, q * r)
    jj = b * sp.spherical_jn(l, q * r) + c * sp.spherical_yn(l, q * r)
    return np.sum(w * z * z * r * r), np.sum(w * z * jj * r * r)


@pytest.mark.parametrize("p2", [0.3 + 0.02j, 0.55 + 0.3j, -0.2 + 0.1j, 0.7 + 0.005j])
@pytest.mark.parametrize("l", [0, 1, 2, 3])
def test_radial_integrals_closed_form(p2, l):
    F, G = S.sqwell_fg(p2, -0.8, 2.5, l)
    Fq, Gq = _fg_quadrature(p2, -0.8, 2.5, l)
    assert abs(F - Fq) < 1e-11 * abs(Fq)
    assert abs(G - Gq) < 1e-11 * abs(Gq)


@pytest.mark.parametrize("l", [0, 1, 2, 3])
def test_single_site_dos_positive(l):
    # isolated well (tau = t) just above the real axis: DOS inside the sphere > 0
    for e in (0.2, 0.45, 0.7):
        p2 = e + 1e-6j
        F, G = S.sqwell_fg(p2, -0.8, 2.5, l)
        ck, q = S.kappa_of(p2), S.kappa_of(p2 + 0.8)
        tand = S._tan_delta(ck, q, 2.5, l)[l]
        t = (-tand / ck) / (1 + 1j * ck * (-tand / ck))
        assert -np.imag(F * t - G) / np.pi > 0


@pytest.mark.parametrize("irel,lmax,para", [(0, 2, True), (0, 3, False), (1, 2, False), (1, 3, False)])
def test_oracle_layer_dos_formula(irel, lmax, para):
    rng = np.random.default_rng(5)
    nd = (2 if irel else 1) * (lmax + 1) ** 2
    nlay = 3
    tau = rng.normal(size=(nlay, nd, nd)) + 1j * rng.normal(size=(nlay, nd, nd))
    F = rng.normal(size=(nlay, nd)) + 1j * rng.normal(size=(nlay, nd))
    G = rng.normal(size=(nlay, nd)) + 1j * rng.normal(size=(nlay, nd))
    zm, zl = O.layer_dos(tau, F, G, lmax, irel, para)
    fac = -1 / np.pi * (2 if para and not irel else 1)
    lv = S.kmy_l_kappa(lmax)[0] if irel else S.lm_l(nd)
    for li in range(nlay):
        ref = fac * (F[li] * np.diag(tau[li]) - G[li])
        assert np.allclose(zm[li], ref, rtol=1e-14, atol=0)
        for l in range(lmax + 1):
            assert abs(zl[li, l] - ref[lv == l].sum()) < 1e-13 * np.abs(ref).sum()


def test_layer_dos_inputs_shapes():
    ep = W.energy_problem(W.rel_bcc(nsets=[2] * 24), 10)
    F, G = S.layer_dos_inputs(ep, "a")
    assert F.shape == (ep.nintfc, ep.lkmax) and np.all(np.isfinite(F)) and np.all(np.isfinite(G))
    # kappa = -1 (l=0, j=1/2) pair shares one radial function
    assert F[0, 0] == F[0, 1]
