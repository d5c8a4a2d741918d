"""Bloch spectral function, host side: the radial overlaps of the model's
wells, the pairing operators of rsp-scf/pairing.f in the (kappa,mu) basis,
and the oracle's restatement of bsf.f (its pure-species and non-CPA limits,
and its agreement with the oracle's layer DOS)."""
import numpy as np
import pytest

import bsf_ref as B
import oracle as O
from skkr_budapest_gb300 import synth as S


@pytest.mark.parametrize("p2,v,l", [(0.65 + 0.24j, -0.8, 0), (0.65 + 0.24j, -0.8, 3), (0.7 + 1e-4j, -1.1, 2),
                                    (0.4 + 0.01j, -0.6, 1)])
def test_overlap_of_one_solution_is_the_layer_dos_integral(p2, v, l):
    z = S.sqwell_regular(p2, v, 2.4, l)
    f, _ = S.sqwell_fg(p2, v, 2.4, l)
    assert abs(S.radial_overlap(z, z, 2.4, l) - f) < 1e-12 * abs(f)


@pytest.mark.parametrize("l", [0, 1, 2, 3])
def test_overlap_of_two_wells_against_the_lommel_form(l):
    """int_0^R j_l(ar) j_l(br) r^2 dr = R^2 (b j_l(aR) j_l'(bR) - a j_l'(aR) j_l(bR)) / (a^2 - b^2)."""
    R = 2.4
    za = S.sqwell_regular(0.62 + 0.05j, -0.9, R, l)
    zb = S.sqwell_regular(0.62 + 0.05j, -0.5, R, l)

    def jd(x):
        j = S.sph_bessel(l + 1, x)[0]
        jm = np.cos(x) / x if l == 0 else j[l - 1]
        return j[l], jm - (l + 1) / x * j[l]

    a, b = za[1], zb[1]
    ja, dja = jd(a * R)
    jb, djb = jd(b * R)
    closed = za[0] * zb[0] * R * R * (b * ja * djb - a * dja * jb) / (a * a - b * b)
    got = S.radial_overlap(za, zb, R, l)
    assert abs(got - closed) < 1e-11 * abs(closed)
    # the hole form conjugates the second solution
    got_h = S.radial_overlap(za, zb, R, l, conj_b=True)
    zbc = (np.conj(zb[0]), np.conj(zb[1]))
    assert abs(got_h - S.radial_overlap(za, zbc, R, l)) < 1e-13 * abs(got_h)


@pytest.mark.parametrize("lmax", [1, 2, 3])
def test_pairing_operators(lmax):
    P = S.pairing_kmy(lmax)
    lv, _ = S.kmy_l_kappa(lmax)
    eps = S.pairing_metric(lmax)
    # pairing.f's singlet is the metric of the BdG t^-1 up to the parity (-1)^(l+1)
    sign = np.where(lv % 2 == 0, -1.0, 1.0)
    assert np.abs(P["singlet"] - 0.5 * sign[:, None] * eps).max() < 1e-14
    # every operator pairs orbitals of the same l with m' = -m: (kappa, mu)
    # with (kappa', -mu) for the unequal-spin ones, mu + mu' = +-1 for the
    # equal-spin triplets
    mu2 = np.zeros(len(lv), int)
    for kap in set(S.kmy_l_kappa(lmax)[1].tolist()):
        idx = np.where(S.kmy_l_kappa(lmax)[1] == kap)[0]
        mu2[idx] = np.arange(-(2 * abs(kap) - 1), 2 * abs(kap), 2)
    for name, m in P.items():
        nz = np.argwhere(np.abs(m) > 1e-13)
        assert len(nz), name
        for i, j in nz:
            want = (0,) if name in ("singlet", "t0") else (-2, 2)
            assert lv[i] == lv[j] and mu2[i] + mu2[j] in want, (name, i, j)
    # equal-spin triplets are built from the spin-diagonal blocks: up and down
    # differ (a sign and a factor i on the down-down block)
    assert np.abs(P["tup"] - P["tdown"]).max() > 0.1


def _rand(rng, n, scale=1.0, diag=0.0):
    return scale * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) + diag * np.eye(n)


@pytest.mark.parametrize("bdg", [False, True])
def test_oracle_pure_species_equals_the_coherent_form(bdg):
    """With tau_A = tau_B = tau_c and one radial function for both species,
    D_a = 1 and A0 + A1 = R tau_c + R (tau(k) - tau_c) = R tau(k) for every
    concentration: the CPA form reduces to the layer without CPA."""
    rng = np.random.default_rng(4)
    nd = 64 if bdg else 32
    nde = nd // 2 if bdg else nd
    tk = _rand(rng, nd, 0.2)
    tc = _rand(rng, nd, 0.2, 3.0)
    f1 = rng.normal(size=nd) + 1j * rng.normal(size=nd)
    F = np.broadcast_to(f1, (2, 2, nd)).copy()
    fe1 = rng.normal(size=(nde, nde)) + 1j * rng.normal(size=(nde, nde))
    Feh = np.broadcast_to(fe1, (2, 2, nde, nde)).copy() if bdg else None
    pair = S.pairing_kmy(3) if bdg else None
    ref = B.bsf_layer(tk, tc, tc, tc, 1.0, F, Feh, pair)
    for c in (0.3, 0.75, 1 - 2e-6):
        got = B.bsf_layer(tk, tc, tc, tc, c, F, Feh, pair)
        assert np.abs(got - ref).max() < 1e-10 * np.abs(ref).max(), c
    if bdg:
        assert np.abs(ref[1:]).max() > 0


def test_oracle_without_cpa_is_the_layer_dos_of_tau_k():
    """A layer without CPA: bsfe = sum over the basis of Im -1/pi F_i tau(k)_ii,
    the oracle's layer DOS (orc_layer_dos) of tau(k) with G = 0."""
    rng = np.random.default_rng(5)
    for irel, lmax in ((1, 3), (0, 2)):
        nd = (2 if irel else 1) * (lmax + 1) ** 2
        tk = _rand(rng, nd, 0.3)
        f = rng.normal(size=nd) + 1j * rng.normal(size=nd)
        F = np.zeros((2, 2, nd), complex)
        F[0, 0] = f
        for para in (False, True):
            got = B.bsf_layer(tk, tk, tk, tk, 1.0, F, para=para, irel=irel)
            _, zl = O.layer_dos(tk[None], f[None], np.zeros((1, nd)), lmax, irel, para)
            assert abs(got[0] - zl.imag.sum()) < 1e-12 * abs(got[0]), (irel, para)
            assert np.all(got[1:] == 0)


def test_radial_overlaps_of_a_system():
    from skkr_budapest_gb300 import workloads as W
    ep = W.energy_problem(W.rel_bcc_cpa(nsets=[4] * 24), 12)
    F, Feh = S.bsf_radial(ep)
    assert Feh is None and F.shape == (ep.nintfc, 2, 2, ep.lkmax)
    # the diagonal species pairs are the layer DOS integrals of each species
    Fa, _ = S.layer_dos_inputs(ep, "a")
    Fb, _ = S.layer_dos_inputs(ep, "b")
    assert np.abs(F[:, 0, 0] - Fa).max() < 1e-11 * np.abs(Fa).max()
    assert np.abs(F[:, 1, 1] - Fb).max() < 1e-11 * np.abs(Fb).max()
    # the cross overlaps are symmetric in the species and differ on alloy layers
    assert np.abs(F[:, 0, 1] - F[:, 1, 0]).max() < 1e-13 * np.abs(F).max()
    alloy = [li for li in range(ep.nintfc) if ep.conc[li] < 1]
    assert alloy and np.abs(F[alloy, 0, 1] - F[alloy, 0, 0]).max() > 1e-3 * np.abs(F).max()


def test_radial_overlaps_of_a_bdg_system():
    from skkr_budapest_gb300 import workloads as W
    ep = W.energy_problem(W.bdg_bcc(nsets=[3] * 64), 30)
    F, Feh = S.bsf_radial(ep)
    nde = ep.lkmax // 2
    assert F.shape == (ep.nintfc, 2, 2, 2 * nde) and Feh.shape == (ep.nintfc, 2, 2, nde, nde)
    lv, _ = S.kmy_l_kappa(ep.lmax)
    off = lv[:, None] != lv[None, :]
    assert np.all(Feh[..., off] == 0) and np.abs(Feh[..., ~off]).min() > 0
    # near E_F the hole solutions (conjugates at psqh ~ conj psq) give
    # overlaps close to the electron ones, conjugated
    assert np.abs(F[:, 0, 0, nde:] - np.conj(F[:, 0, 0, :nde])).max() < 1e-2 * np.abs(F).max()


def oracle_bsf_chain(ep, kpts, cpa):
    """The oracle's chain for the spectral function of bsf.f: the converged
    CPA (m_c, tau_c, tau_A, tau_B) of `cpa`, a one-point k loop per k point on
    m_c (identity alone, no alloy), phystau of every tau, then bsf_layer per
    layer.  Returns [nk, nintfc, 6]."""
    import dataclasses
    mc = cpa["tminv"]
    lay = range(ep.nintfc)

    def phys(tau, tinv):
        return np.array([O.phystau(tau[li], tinv[li], ep.alpha[li], ep.lmax, ep.irel) for li in lay])

    tc, ta, tb = phys(cpa["tauc"], mc), phys(cpa["taua"], ep.tminva), phys(cpa["taub"], ep.tminvb)
    one = dataclasses.replace(ep, lg=ep.lg[:1], rg=ep.rg[:1], conc=np.ones(ep.nintfc), tminv=mc.copy(),
                              tminva=mc.copy(), tminvb=mc.copy())
    F, Feh = S.bsf_radial(ep)
    pair = S.pairing_kmy(ep.lmax) if ep.irel == 2 else None
    out = []
    for k in np.asarray(kpts, float).reshape(-1, 2):
        r = O.cpacoord(one.with_k(k[None, :], np.ones(1)))
        assert r["status"] == 0 and r["cpa_iterations"] == 1
        tk = phys(r["tauc"], mc)
        out.append([B.bsf_layer(tk[li], tc[li], ta[li], tb[li], ep.conc[li], F[li],
                                None if Feh is None else Feh[li], pair, irel=ep.irel) for li in lay])
    return np.array(out)


def small_cpa_problem():
    from skkr_budapest_gb300 import workloads as W
    spec = W.rel_bcc_cpa(nsets=[2] * 24)
    spec.lmax = 1
    return W.energy_problem(spec, 16, kmesh="full")


def test_cpa_form_integrates_to_the_component_dos():
    """Over the full zone sum_k w_k (tau(k) - tau_c) = 0, so the k average of
    the CPA form is A0 = -1/pi Im sum_a c_a sum_i F^aa_i tau_a,ii, the
    concentration-weighted component DOS (without the irregular term), and a
    layer without CPA averages to -1/pi Im sum_i F_i tau_c,ii."""
    ep = small_cpa_problem()
    assert abs(ep.wk.sum() - 1.0) < 1e-12 and any(c < 1 for c in ep.conc)
    cpa = O.cpacoord(ep)
    assert cpa["status"] == 0 and cpa["cpa_iterations"] > 1
    a = oracle_bsf_chain(ep, ep.xk, cpa)
    avg = np.tensordot(ep.wk, a[:, :, 0], axes=([0], [0]))
    F, _ = S.bsf_radial(ep)
    mc = cpa["tminv"]
    for li in range(ep.nintfc):
        def ph(t, ti):
            return O.phystau(t[li], ti[li], ep.alpha[li], ep.lmax, ep.irel)
        if ep.conc[li] < 1:
            c = ep.conc[li]
            want = c * np.sum(F[li, 0, 0] * np.diag(ph(cpa["taua"], ep.tminva))) + \
                (1 - c) * np.sum(F[li, 1, 1] * np.diag(ph(cpa["taub"], ep.tminvb)))
        else:
            want = np.sum(F[li, 0, 0] * np.diag(ph(cpa["tauc"], mc)))
        want = (-want / np.pi).imag
        assert abs(avg[li] - want) < 1e-7 * abs(want), (li, avg[li], want)
