"""Bloch spectral function with its CPA and BdG forms on the device
(skkr_gpu_bsf, api.bsf) against the oracle's restatement of bsf.f: the
device sums on random taus of every mode with CPA and plain layers mixed,
then the whole chain (CPA of the energy, one-point k loops on m_c, phystau,
skkr_gpu_bsf) on an alloy interface and on the BdG interface, and the
k-average identity of the CPA form on the device."""
import numpy as np
import pytest

import bsf_ref as B
import oracle as O
from skkr_budapest_gb300 import native as N
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W
from test_bsf import oracle_bsf_chain, small_cpa_problem

pytestmark = pytest.mark.gpu


def _rand(rng, shape, scale=1.0):
    return scale * (rng.normal(size=shape) + 1j * rng.normal(size=shape))


@pytest.mark.parametrize("mode,lmax,para", [(1, 3, False), (2, 3, False), (0, 2, True), (2, 1, False)])
def test_device_sums_match_the_oracle(mode, lmax, para):
    rng = np.random.default_rng(10 + mode)
    nd = {0: 1, 1: 2, 2: 4}[mode] * (lmax + 1) ** 2
    nde = nd // 2 if mode == 2 else nd
    nk, nlay = 5, 4
    conc = np.array([1.0, 0.35, 0.8, 1.0])
    eye = np.eye(nd)
    tk = _rand(rng, (nk, nlay, nd, nd), 0.2)
    tc = _rand(rng, (nlay, nd, nd), 0.2) + 2.5 * eye
    ta = _rand(rng, (nlay, nd, nd), 0.2) + 2.0 * eye
    tb = _rand(rng, (nlay, nd, nd), 0.2) + 3.0 * eye
    F = _rand(rng, (nlay, 2, 2, nd))
    Feh = _rand(rng, (nlay, 2, 2, nde, nde)) if mode == 2 else None
    P = S.pairing_kmy(lmax) if mode == 2 else None
    pair = None if P is None else np.array([P[x] for x in B.PAIRS])
    got = N.bsf(mode, lmax, conc, tk, tc, ta, tb, F, Feh, pair, para)
    ref = np.array([[B.bsf_layer(tk[k, l], tc[l], ta[l], tb[l], conc[l], F[l], None if Feh is None else Feh[l], P,
                                 para=para, irel=mode) for l in range(nlay)] for k in range(nk)])
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(got - ref).max() < 1e-11 * scale, np.abs(got - ref).max() / scale
    if mode != 2:
        assert np.all(got[:, :, 1:] == 0)


def test_cpa_chain_matches_the_oracle():
    """Alloy interface (relativistic, lmax = 1, four alloy layers): the
    device chain from its own CPA against the oracle chain from the
    oracle's CPA; the two CPAs agree to their tolerance, 1e-10."""
    from skkr_budapest_gb300 import api
    ep = small_cpa_problem()
    kpts = [(0.0, 0.0), (0.31, 0.12), (0.5, 0.5)]
    got = api.bsf(ep, kpts)
    ref = oracle_bsf_chain(ep, kpts, O.cpacoord(ep))[:, :, 0]
    assert set(got) == {"bsfe"}
    assert np.abs(got["bsfe"] - ref).max() < 1e-8 * np.abs(ref).max()


def test_cpa_form_integrates_to_the_component_dos_on_the_device():
    from skkr_budapest_gb300 import api
    ep = small_cpa_problem()
    cpa = api.cpacoord(ep)
    a = api.bsf(ep, ep.xk, cpa=cpa)["bsfe"]
    avg = np.tensordot(ep.wk, a, axes=([0], [0]))
    F, _ = S.bsf_radial(ep)
    for li in range(ep.nintfc):
        def ph(t, ti):
            return N.phystau(t[li], ti[li], ep.alpha[li], ep.lmax, ep.irel)
        if ep.conc[li] < 1:
            c = ep.conc[li]
            want = c * np.sum(F[li, 0, 0] * np.diag(ph(cpa["taua"], ep.tminva))) + \
                (1 - c) * np.sum(F[li, 1, 1] * np.diag(ph(cpa["taub"], ep.tminvb)))
        else:
            want = np.sum(F[li, 0, 0] * np.diag(ph(cpa["tauc"], cpa["tminv"])))
        want = (-want / np.pi).imag
        assert abs(avg[li] - want) < 1e-7 * abs(want), (li, avg[li], want)


def test_bdg_chain_matches_the_oracle():
    """BdG interface (lmax = 1, superconducting half): the six components of
    bsf.f per layer against the oracle chain."""
    from skkr_budapest_gb300 import api
    spec = W.bdg_bcc(nsets=[2] * 64, lmax=1)
    ep = W.energy_problem(spec, 30)
    kpts = [(0.0, 0.0), (0.4, 0.2)]
    got = api.bsf(ep, kpts)
    ref = oracle_bsf_chain(ep, kpts, O.cpacoord(ep))
    assert set(got) == set(api.BSF_NAMES)
    scale = np.abs(ref).max()
    for i, name in enumerate(api.BSF_NAMES):
        assert np.abs(got[name] - ref[:, :, i]).max() < 1e-9 * scale, name
    # singlet pairing without spin-orbit coupling: the singlet component is
    # there, the triplet components vanish
    eh = np.abs(got["bsfeh"])
    assert eh.max() > 1e-4 * scale
    for name in ("bsfhe", "bsfteh", "bsfthe"):
        assert np.abs(got[name]).max() < 1e-12 * eh.max(), name
