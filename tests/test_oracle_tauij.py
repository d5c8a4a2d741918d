"""Off-diagonal tau of the interface (skkr_dbogo_bsf/clu/tau2d_god.f and the
pair k sums of skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:760-840) in the oracle:
every layer-pair block of the full Godfrin tau equals the block of a direct
inverse of a long finite slab, the IBZ sum with group rotations and phases
equals the sum over the full Brillouin zone, and the on-site pair is the
layer-diagonal k sum."""
import numpy as np
import pytest
from scipy.linalg import solve_banded

import oracle as O
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W


def _slab_columns(ep, k, nb=150):
    g = O.gk_blocks(ep.rt, k)
    lk, pl, nprc, jm = ep.lkmax, int(ep.ninprc[1]), ep.nprc, ep.rt.jmax
    nlay = pl * (nprc + 2 * nb)
    ntot = nlay * lk
    bw = (jm + 1) * lk - 1
    ab = np.zeros((2 * bw + 1, ntot), complex)

    def put(i0, j0, blk):
        for a in range(lk):
            for b in range(lk):
                ab[bw + i0 + a - (j0 + b), j0 + b] += blk[a, b]

    for i in range(nlay):
        li = i - nb * pl
        put(i * lk, i * lk, ep.tminv[li] if 0 <= li < ep.nintfc else ep.tminvl[0])
        for j in range(-jm, jm + 1):
            b = ep.rt.blk_of_j.get(j)
            if b is not None and 0 <= i + j < nlay:
                put(i * lk, (i + j) * lk, -g[b])
    rhs = np.zeros((ntot, ep.nintfc * lk), complex)
    c0 = nb * pl * lk
    rhs[c0:c0 + ep.nintfc * lk, :] = np.eye(ep.nintfc * lk)
    return solve_banded((bw, bw), ab, rhs)[c0:c0 + ep.nintfc * lk]


def test_full_godfrin_tau_equals_slab_inverse():
    ep = W.energy_problem(W.plain_fcc(nset=2), 5)
    t = O.tau2dgod_k(ep, 0)
    cols = _slab_columns(ep, ep.xk[0])
    lk, n = ep.lkmax, ep.nintfc
    for a in range(n):
        for b in range(n):
            blk = cols[a * lk:(a + 1) * lk, b * lk:(b + 1) * lk]
            assert np.linalg.norm(blk - t[a, b]) < 1e-12 * np.linalg.norm(blk), (a, b)


def c4v_a0mat():
    # the in-plane part of g^T for the operations whose rotations are
    # point_group_mats (L_g = D(g)): k of the wedge stands for g k of the BZ
    return [o[:2, :2].T.ravel() for o in S.c4v_ops()]


def _pairs_and_positions(spec, ep):
    a2d = spec.stacking.a2d
    l0 = int(ep.ninprc[0])
    cvec = np.array([[0.5 * ((l0 + l) % 2) * a2d] * 2 for l in range(ep.nintfc)])
    n = ep.nintfc
    pairs = [(0, 0, 0, 1), (1, 0, 0, 0), (1, 1, 2, 3 % n), (0, -1, 3 % n, 1), (2, 1, 1, (4 % n)), (0, 0, 2, 2)]
    return pairs, [a2d, 0.0], [0.0, a2d], cvec


@pytest.mark.parametrize("kind", ["plain", "rel"])
def test_ibz_pair_sums_equal_full_zone(kind):
    if kind == "plain":
        spec, ie = W.plain_fcc(nset=4), 4
    else:
        spec = W.rel_bcc(nsets=[3] * 24)
        spec.lmax = 1
        ie = 16
    ep = W.energy_problem(spec, ie)
    epf = W.energy_problem(spec, ie, kmesh="full")
    pairs, a1, a2, cvec = _pairs_and_positions(spec, ep)
    r = O.tauij(ep, pairs, a1, a2, cvec, c4v_a0mat(), nthreads=4)
    rf = O.tauij(epf, pairs, a1, a2, cvec, [np.eye(2).ravel()], nthreads=4)
    assert r["status"] == 0 and rf["status"] == 0
    for q in range(len(pairs)):
        for key in ("tau_ij", "tau_ji"):
            d = np.linalg.norm(r[key][q] - rf[key][q]) / np.linalg.norm(rf[key][q])
            assert d < 1e-11, (kind, key, pairs[q], d)
    # the on-site pair is the layer-diagonal k sum of cpacoord
    assert np.array_equal(r["tau_ij"][5], r["tauc"][2])
    c = O.cpacoord(ep, nthreads=4)
    assert np.linalg.norm(r["tauc"] - c["tauc"]) < 1e-13 * np.linalg.norm(c["tauc"])
