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


@pytest.mark.parametrize("irel,lmax", [(0, 2), (1, 3), (2, 2)])
def test_phystau2_matches_oracle(irel, lmax):
    # pair block screened -> physical (phystau2.f, idiag = 0), two layers'
    # screening on the two sides
    rng = np.random.default_rng(17 + irel)
    lm = (lmax + 1) ** 2
    nd = lm if irel == 0 else 2 * lm if irel == 1 else 4 * lm
    nal = lmax + 1 if irel < 2 else 2 * (lmax + 1)
    c = lambda *s: rng.normal(size=s) + 1j * rng.normal(size=s)
    tau, t1, t2, a1, a2 = c(nd, nd), c(nd, nd), c(nd, nd), 0.3 * c(nal), 0.3 * c(nal)
    g = native.phystau2(tau, t1, a1, t2, a2, lmax, irel)
    o = O.phystau2(tau, t1, a1, t2, a2, lmax, irel)
    assert np.linalg.norm(g - o) < 1e-12 * np.linalg.norm(o)


def test_host_tau_file_matches_oracle(tmp_path):
    # cpacoord, then the pair sums with its coherent t^-1, then the physical
    # tau of every pair and layer into the .tau file the cluster code reads
    # (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:949-1036); read back and
    # compared with the oracle's chain
    from skkr_budapest_gb300 import tauh
    ep, pairs, a1, a2, cvec, a0mat = _case("plain")
    ctx = api.Context.for_problem(ep, "fp64")
    try:
        r = ctx.cpacoord(ep)
    finally:
        ctx.close()
    ctx = api.Context.for_problem(ep, "fp64")
    try:
        t = ctx.tauij(ep, pairs, a1, a2, cvec, a0mat, tminv=r["tminv"])
    finally:
        ctx.close()
    path = api.write_host_tau(str(tmp_path / "host"), 5, ep, r["tminv"], r["tauc"], t, pairs)
    assert path.endswith("host0005.tau")
    f = tauh.read_tauh(str(tmp_path / "host"), 5, ep.ce, pairs, ep.nintfc, ep.lkmax)
    assert f["nk"] == ep.nk
    o = O.tauij(ep, pairs, a1, a2, cvec, a0mat, tminv=r["tminv"], nthreads=8)
    tm, al = r["tminv"], ep.alpha
    for q, (_, _, i, j) in enumerate(pairs):
        w_ij = O.phystau2(o["tau_ij"][q], tm[i], al[i], tm[j], al[j], ep.lmax, ep.irel)
        w_ji = O.phystau2(o["tau_ji"][q], tm[j], al[j], tm[i], al[i], ep.lmax, ep.irel)
        assert np.linalg.norm(f["tau_ij"][q] - w_ij) < 1e-10 * np.linalg.norm(w_ij), pairs[q]
        assert np.linalg.norm(f["tau_ji"][q] - w_ji) < 1e-10 * np.linalg.norm(w_ji), pairs[q]
    for li in range(ep.nintfc):
        w = O.phystau(r["tauc"][li], tm[li], al[li], ep.lmax, ep.irel)
        assert np.linalg.norm(f["tau_ii"][li] - w) < 1e-12 * np.linalg.norm(w), li
