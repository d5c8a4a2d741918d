"""The benchmarked workload itself against the oracle: the relativistic
bcc(001) PL4 lmax=3 interface (n_PL = 128) at its own contour energies and
meshes, k-strided so that the oracle finishes in seconds.  Energies 12, 19
and 23 have 528, 2485 and 12090 k points and Im E = 0.24, 0.022 and 5e-4
Ry; at 23 the split-precision path runs its near-axis policy (7-slice
exact-level products, split-precision decimation).  FP64 path: relative
Frobenius error <= 1e-10 on the k-summed tau with the oracle's decimation
iteration counts; split-precision path: <= 1e-9."""
import os

import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import api
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# (contour energy, k stride): every stride-th point of the IBZ list, from the
# first to the last, covers the whole zone
CASES = [(12, 10), (19, 40), (23, 40)]
_oracle_cache = {}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _problem(ie, stride):
    ep = W.energy_problem(W.rel_bcc(), ie)
    idx = np.arange(0, ep.nk, stride)
    return ep, ep.with_k(ep.xk[idx], ep.wk[idx] / ep.wk[idx].sum())


def _oracle(ie, stride):
    if (ie, stride) not in _oracle_cache:
        _, sub = _problem(ie, stride)
        _oracle_cache[(ie, stride)] = O.cpacoord(sub, nthreads=os.cpu_count() or 1)
    return _oracle_cache[(ie, stride)]


@pytest.mark.parametrize("ie,stride", CASES)
def test_fp64_path_on_the_benchmarked_meshes(ie, stride):
    ep, sub = _problem(ie, stride)
    assert ep.nk == [528, 2485, 12090][[12, 19, 23].index(ie)]
    o = _oracle(ie, stride)
    g = api.cpacoord(sub, precision="fp64")
    assert o["status"] == 0 and g["status"] == 0
    assert g["max_dec_iters"] == o["max_dec_iters"]
    assert g["cpa_iterations"] == o["cpa_iterations"]
    for key in ("tauc", "taua", "taub"):
        assert rel(g[key], o[key]) < 1e-10, (key, rel(g[key], o[key]))


@pytest.mark.parametrize("ie,stride", CASES)
def test_split_precision_path_on_the_benchmarked_meshes(ie, stride):
    _, sub = _problem(ie, stride)
    o = _oracle(ie, stride)
    g = api.cpacoord(sub, precision="mixed")
    assert g["status"] == 0
    err = rel(g["tauc"], o["tauc"])
    assert err < 1e-9, err
    assert g["max_refine_resid"] < 1e-6
