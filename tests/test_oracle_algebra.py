"""Algebraic identities of the oracle's restated routines (CPU)."""
import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W

rng = np.random.default_rng(7)


def crand(*shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def test_gjinv_inverse_and_logdet():
    for n in (1, 5, 18, 40):
        a = crand(n, n) + 3 * np.eye(n)
        inv, detl = O.gjinv(a)
        assert np.linalg.norm(inv @ a - np.eye(n)) < 1e-11 * n
        sign, logabs = np.linalg.slogdet(a)
        assert abs(np.exp(detl) - sign * np.exp(logabs)) < 1e-8 * abs(np.exp(logabs))


def test_relmtrx_is_clebsch_transform():
    lmax = 3
    lm = (lmax + 1) ** 2
    a = crand(lm, lm)
    fac = 1.0003 + 0.0001j
    b = O.relmtrx(a, fac, lmax)
    U = S.clebsch_u(lmax)
    ref = U.T @ np.kron(np.eye(2), fac * a) @ U
    assert np.allclose(b, ref, atol=1e-13)


def test_surfgfd_fixed_point():
    # semi-infinite chain: X^-1 = m0 - ml X^-1 mr  for the decimated x
    n = 12
    m0 = crand(n, n) * 0.3 + (2.0 + 1.0j) * np.eye(n)
    ml = crand(n, n) * 0.2
    mr = crand(n, n) * 0.2
    x, st, it = O.surfgfd(ml, m0, mr, itermax=60, errmax=1e-13)
    assert st == 0 and it < 60
    xinv = np.linalg.inv(x)
    assert np.linalg.norm(xinv - (m0 - ml @ x @ mr)) < 1e-10 * np.linalg.norm(xinv)


def test_tau2d_equals_direct_inverse_of_slab():
    # tau2d diagonal blocks == blocks of the inverse of a long finite slab
    # (the semi-infinite leads replaced by 150 bulk principal layers per side)
    from scipy.linalg import solve_banded
    spec = W.plain_fcc(nset=2)
    ep = W.energy_problem(spec, 5)
    r = O.cpacoord(ep.with_k(ep.xk[:1], np.array([1.0])), nthreads=1)
    k = ep.xk[0]
    g = O.gk_blocks(ep.rt, k)
    lk, pl, nprc, jm = ep.lkmax, int(ep.ninprc[1]), ep.nprc, ep.rt.jmax
    nb = 150
    nlay = pl * (nprc + 2 * nb)
    ntot = nlay * lk
    bw = (jm + 1) * lk - 1
    ab = np.zeros((2 * bw + 1, ntot), complex)

    def put(i0, j0, blk):
        for a in range(lk):
            for b in range(lk):
                ii, jj = i0 + a, j0 + b
                ab[bw + ii - jj, jj] += blk[a, b]

    for i in range(nlay):
        li = i - nb * pl
        t = ep.tminv[li] if 0 <= li < ep.nintfc else ep.tminvl[0]
        put(i * lk, i * lk, t)
        for j in range(-jm, jm + 1):
            b = ep.rt.blk_of_j.get(j)
            if b is not None and 0 <= i + j < nlay:
                put(i * lk, (i + j) * lk, -g[b])
    rhs = np.zeros((ntot, ep.nintfc * lk), complex)
    c0 = nb * pl * lk
    rhs[c0:c0 + ep.nintfc * lk, :] = np.eye(ep.nintfc * lk)
    cols = solve_banded((bw, bw), ab, rhs)
    ngeff = len(ep.lg)
    for li in range(ep.nintfc):
        i = c0 + li * lk
        blk = cols[i:i + lk, li * lk:(li + 1) * lk]
        avg = sum(ep.lg[q] @ blk @ ep.rg[q] for q in range(ngeff)) / ngeff
        err = np.linalg.norm(avg - r["tauc"][li]) / np.linalg.norm(avg)
        assert err < 1e-9, (li, err)


def test_cpa_condition_at_convergence():
    # converged CPA: c tau_A + (1-c) tau_B = tau_c on every alloy layer
    spec = W.plain_fcc(nset=3)
    spec.alloy_layers = (2, 3)
    spec.seed = 11
    ep = W.energy_problem(spec, 6)
    r = O.cpacoord(ep, nthreads=2)
    assert r["status"] == 0
    assert 1 < r["cpa_iterations"] < ep.itcpam
    assert r["cpa_error"] <= ep.cpatol
    for li in (2, 3):
        c = ep.conc[li]
        lhs = c * r["taua"][li] + (1 - c) * r["taub"][li]
        assert np.linalg.norm(lhs - r["tauc"][li]) < 1e-8 * np.linalg.norm(r["tauc"][li])


def test_threaded_k_split_matches_serial():
    spec = W.plain_fcc(nset=4)
    ep = W.energy_problem(spec, 3)
    r1 = O.cpacoord(ep, nthreads=1)
    r3 = O.cpacoord(ep, nthreads=3)
    assert np.linalg.norm(r1["tauc"] - r3["tauc"]) < 1e-13 * np.linalg.norm(r1["tauc"])


@pytest.mark.parametrize("kind", ["plain", "rel"])
def test_full_bz_equals_symmetrised_ibz(kind):
    if kind == "plain":
        spec = W.plain_fcc(nset=4)
        ie = 4
    else:
        spec = W.rel_bcc(nsets=[3] * 24)
        spec.lmax = 2  # keep the CPU case small: (kappa,mu) 18/site
        ie = 16
    ep = W.energy_problem(spec, ie)
    epf = W.energy_problem(spec, ie, kmesh="full")
    r = O.cpacoord(ep, nthreads=2)
    rf = O.cpacoord(epf, nthreads=2)
    assert r["status"] == 0 and rf["status"] == 0
    d = np.linalg.norm(rf["tauc"] - r["tauc"]) / np.linalg.norm(r["tauc"])
    assert d < 1e-9
