"""BdG path (skkr_dbogo_bsf layout, SKKR_BDG) on the GPU against the oracle:
the full k-summed tau and its electron-hole (anomalous) block at <= 1e-10 on
the FP64 path, at the C5 size (lmax=3, n_s=64, PL4: n_PL=256, Im E=1e-4) and
on a small lmax=1 stack; the split-precision path (electron-first layout,
products split into electron and hole K halves) against FP64 at <= 1e-9 on
the full tau and on the anomalous block alone."""
import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import api, native
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _check(g, o, km):
    assert g["status"] == 0 and o["status"] == 0
    assert g["max_dec_iters"] == o["max_dec_iters"]
    assert rel(g["tauc"], o["tauc"]) < TOL, rel(g["tauc"], o["tauc"])
    eh = (slice(None), slice(0, km), slice(km, 2 * km))
    assert rel(g["tauc"][eh], o["tauc"][eh]) < TOL, rel(g["tauc"][eh], o["tauc"][eh])


@pytest.mark.parametrize("ie", [0, 2])
def test_bdg_small_stack(ie):
    ep = W.energy_problem(W.bdg_bcc(lmax=1, pl=2, ne=4, im_e=1e-2), ie, nset=3)
    _check(api.cpacoord(ep), O.cpacoord(ep, nthreads=8), ep.lkmax // 2)


@pytest.mark.parametrize("ie", [5, 30])
def test_bdg_c5_size(ie):
    ep = W.energy_problem(W.bdg_bcc(), ie, nset=2)
    assert ep.n_pl == 256
    _check(api.cpacoord(ep), O.cpacoord(ep, nthreads=16), ep.lkmax // 2)


@pytest.mark.parametrize("ie,im_e", [(10, 5e-3), (50, 5e-3), (10, 5e-4)])
def test_bdg_mixed_against_fp64(ie, im_e):
    # Im E >= 1e-3: decimation runs on the split-precision engine too;
    # closer to the axis it stays in FP64 and only tau2d is split precision
    ep = W.energy_problem(W.bdg_bcc(im_e=im_e), ie, nset=2)
    a = api.cpacoord(ep)
    b = api.cpacoord(ep, precision="mixed")
    km = ep.lkmax // 2
    assert rel(b["tauc"], a["tauc"]) < 1e-9
    assert rel(b["tauc"][:, :km, km:], a["tauc"][:, :km, km:]) < 1e-9


def test_bdg_phystau():
    ep = W.energy_problem(W.bdg_bcc(lmax=2, pl=2, ne=4), 1, nset=1)
    rng = np.random.default_rng(7)
    n = ep.lkmax
    tau = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    g = native.phystau(tau, ep.tminv[0], ep.alpha[0], ep.lmax, 2)
    o = O.phystau(tau, ep.tminv[0], ep.alpha[0], ep.lmax, 2)
    assert rel(g, o) < 1e-12
