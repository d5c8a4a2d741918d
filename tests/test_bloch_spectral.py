"""Bloch spectral function of layers without an alloy (rsp-scf/bsf.f with
the coherent tau): the oracle's chain (one-point k loops with the identity,
phystau, -1/pi Im F tau) integrates over the full-zone mesh to the F part of
the layer DOS of the k-summed tau (CPU).  The device chain
(api.bloch_spectral) against it: test_zz_spectral_gpu.py."""
import dataclasses

import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W


def _oracle_bsf(ep, kpts, para):
    one = dataclasses.replace(ep, lg=ep.lg[:1], rg=ep.rg[:1])
    F, _ = S.layer_dos_inputs(ep, "a")
    out = []
    for k in np.asarray(kpts, float).reshape(-1, 2):
        r = O.cpacoord(one.with_k(k[None, :], np.ones(1)))
        assert r["status"] == 0
        phys = np.array([O.phystau(r["tauc"][li], r["tminv"][li], ep.alpha[li], ep.lmax, ep.irel)
                         for li in range(ep.nintfc)])
        zm, zl = O.layer_dos(phys, F, np.zeros_like(F), ep.lmax, ep.irel, para)
        out.append(zl.imag)
    return np.array(out)


@pytest.mark.parametrize("kind", ["plain", "rel"])
def test_bsf_integrates_to_the_layer_dos(kind):
    if kind == "plain":
        ep = W.energy_problem(W.plain_fcc(nset=4), 8, kmesh="full")
        para = True
    else:
        spec = W.rel_bcc(nsets=[2] * 24)
        spec.lmax = 1
        ep = W.energy_problem(spec, 16, kmesh="full")
        para = False
    assert abs(ep.wk.sum() - 1.0) < 1e-12
    a = _oracle_bsf(ep, ep.xk, para)
    summed = np.tensordot(ep.wk, a, axes=([0], [0]))
    c = O.cpacoord(ep)
    F, _ = S.layer_dos_inputs(ep, "a")
    phys = np.array([O.phystau(c["tauc"][li], c["tminv"][li], ep.alpha[li], ep.lmax, ep.irel)
                     for li in range(ep.nintfc)])
    _, zl = O.layer_dos(phys, F, np.zeros_like(F), ep.lmax, ep.irel, para)
    assert np.abs(summed - zl.imag).max() < 1e-10 * np.abs(zl.imag).max()
