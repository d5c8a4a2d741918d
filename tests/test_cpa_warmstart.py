"""Learned CPA warm start: the committed models load, their features have the
trained shape, and the start they give is a finite kappa-diagonal matrix on
alloy layers only (the CPA loop itself is unchanged)."""
import os

import numpy as np
import pytest

from skkr_budapest_gb300 import cpa_warmstart as CW
from skkr_budapest_gb300 import workloads as W

HERE = os.path.dirname(CW.__file__)


@pytest.mark.parametrize("name", ["cpa_mlp_bcc_lmax3.npz", "cpa_mlp_bcc_lmax3_cont.npz"])
def test_model_start_is_diagonal_on_alloy_layers(name):
    model = CW.Model(os.path.join(HERE, "data", name))
    ep = W.energy_problem(CW._spec(9001), 6, nset=2)
    groups = CW.kappa_groups(ep.lmax)
    nf = 3 + 4 * len(groups) + (2 * len(groups) if model.cont else 0)
    assert model.xmean.shape == (nf,)
    tm = CW.warm_start(ep, model)
    alloy = [li for li in range(ep.nintfc) if 1e-6 < ep.conc[li] < 1 - 1e-6]
    assert alloy
    for li in range(ep.nintfc):
        if li in alloy:
            assert np.all(np.isfinite(tm[li]))
            assert np.abs(tm[li] - np.diag(np.diag(tm[li]))).max() == 0.0
            # a correction of the ATA start, small relative to |m_A - m_B|
            ata, scale = CW._ata_kdiag(ep, li, groups)
            corr = (CW._kdiag(tm[li], groups) - ata) / scale
            assert np.abs(corr).max() < 0.5
        else:
            assert np.array_equal(tm[li], ep.tminv[li])


def test_ata_has_zero_target():
    ep = W.energy_problem(CW._spec(9002), 3, nset=2)
    groups = CW.kappa_groups(ep.lmax)
    li = [l for l in range(ep.nintfc) if 1e-6 < ep.conc[l] < 1 - 1e-6][0]
    assert np.abs(CW.layer_target(ep, li, ep.tminv[li], groups)).max() < 1e-12


def test_host_training_writes_a_model(tmp_path):
    pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    n = 240
    x = rng.normal(size=(n, 11))
    y = 0.3 * np.tanh(x[:, :6] @ rng.normal(size=(6, 6)))
    meta = np.c_[np.repeat(np.arange(12), n // 12), np.zeros(n), np.zeros(n), np.ones(n)]
    data = tmp_path / "d.npz"
    np.savez(data, x=x, y=y, meta=meta, lmax=1)
    out = tmp_path / "m.npz"
    tr, vl, ata = CW.train(str(data), str(out), hidden=16, epochs=200)
    assert np.isfinite(tr) and vl < ata
    model = CW.Model(str(out))
    assert model.predict(x[:3]).shape == (3, 6)
