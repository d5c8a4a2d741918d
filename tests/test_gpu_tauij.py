"""Off-diagonal tau of the interface on the GPU (skkr_gpu_tauij) against the
oracle's restatement of tau2d_god.f and the pair k sums
(skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:760-840): FP64 at 1e-10, the split-
precision path at 1e-9 of the largest pair block."""
import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import api, native
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _case(kind):
    if kind == "plain":
        spec, ie = W.plain_fcc(nset=4), 4
    else:
        spec = W.rel_bcc(nsets=[3] * 24)
        spec.lmax = 1
        ie = 16
    ep = W.energy_problem(spec, ie)
    a2d = spec.stacking.a2d
    l0 = int(ep.ninprc[0])
    n = ep.nintfc
    cvec = np.array([[0.5 * ((l0 + l) % 2) * a2d] * 2 for l in range(n)])
    pairs = [(0, 0, 0, 1), (1, 0, 0, 0), (1, 1, 2, 3), (0, -1, 3, 1), (2, 1, 1, 4), (0, 0, 2, 2), (0, 0, 0, n - 1)]
    a0mat = [o[:2, :2].T.ravel() for o in S.c4v_ops()]
    return ep, pairs, [a2d, 0.0], [0.0, a2d], cvec, a0mat


@pytest.mark.parametrize("kind", ["plain", "rel"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tauij_matches_oracle(kind, precision):
    ep, pairs, a1, a2, cvec, a0mat = _case(kind)
    o = O.tauij(ep, pairs, a1, a2, cvec, a0mat, nthreads=8)
    assert o["status"] == 0
    ctx = api.Context.for_problem(ep, precision)
    try:
        g = ctx.tauij(ep, pairs, a1, a2, cvec, a0mat)
    finally:
        ctx.close()
    assert g["status"] == 0 and g["gpu_launches"] > 0
    scale = max(np.linalg.norm(o["tau_ij"][q]) for q in range(len(pairs)))
    for key in ("tau_ij", "tau_ji"):
        for q in range(len(pairs)):
            d = np.linalg.norm(g[key][q] - o[key][q])
            if precision == "fp64":
                assert d < 1e-10 * np.linalg.norm(o[key][q]), (key, pairs[q], d / np.linalg.norm(o[key][q]))
            else:
                assert d < 1e-9 * scale, (key, pairs[q], d / scale)


def test_tauij_rejects_bad_pairs():
    ep, pairs, a1, a2, cvec, a0mat = _case("plain")
    ctx = api.Context.for_problem(ep, "fp64")
    try:
        with pytest.raises(native.SkkrError):
            ctx.tauij(ep, [(0, 0, 0, ep.nintfc)], a1, a2, cvec, a0mat)
    finally:
        ctx.close()
