"""Bloch spectral function on the device (api.bloch_spectral: one-point k
loops of skkr_gpu_cpacoord with the identity, phystau and the layer-DOS
kernel) against the oracle's chain of test_bloch_spectral.py, 1e-10."""
import numpy as np
import pytest

from skkr_budapest_gb300 import workloads as W
from test_bloch_spectral import _oracle_bsf

pytestmark = pytest.mark.gpu


def test_bsf_on_the_device_matches_the_oracle():
    from skkr_budapest_gb300 import api
    ep = W.energy_problem(W.plain_fcc(nset=4), 8)
    kpts = [(0.0, 0.0), (0.3, 0.1), (0.65, 0.65), (0.2, 0.5)]
    al, _ = api.bloch_spectral(ep, kpts, para=True)
    ref = _oracle_bsf(ep, kpts, True)
    assert np.abs(al - ref).max() < 1e-10 * np.abs(ref).max()


def test_bsf_refuses_alloy_layers():
    from skkr_budapest_gb300 import api
    ep = W.energy_problem(W.rel_bcc_cpa(nsets=[2] * 24), 6)
    with pytest.raises(ValueError):
        api.bloch_spectral(ep, [(0.1, 0.1)])
