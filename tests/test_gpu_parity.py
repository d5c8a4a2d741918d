"""GPU path against the CPU oracle on the same seeded inputs (FP64 path:
relative Frobenius error <= 1e-10 on k-summed tau, species tau and the
converged coherent t-matrix)."""
import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import api, native
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10
rng = np.random.default_rng(3)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n", [1, 9, 18, 54, 128, 256, 448])
def test_gjinv_batch(n):
    a = rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n)) + 2 * np.eye(n)
    g = native.gjinv_batch(a)
    for b in range(3):
        o, _ = O.gjinv(a[b])
        assert rel(g[b], o) < 1e-11


def test_gk_transform():
    ep = W.energy_problem(W.plain_fcc(nset=5), 3)
    g = native.gk(ep.rt, ep.blkmap, ep.lmax, ep.xk)
    for ik in range(ep.nk):
        o = O.gk_blocks(ep.rt, ep.xk[ik])
        assert rel(g[ik], o) < 1e-13


def test_surfgf_batch_matches_oracle():
    n = 20
    m0 = rng.normal(size=(4, n, n)) * 0.3 + (2.0 + 1.0j) * np.eye(n)
    ml = (rng.normal(size=(4, n, n)) + 1j * rng.normal(size=(4, n, n))) * 0.15
    mr = (rng.normal(size=(4, n, n)) + 1j * rng.normal(size=(4, n, n))) * 0.15
    x, st, it = native.surfgf_batch(ml, m0, mr, itermax=50, errmax=1e-10)
    for b in range(4):
        xo, so, io = O.surfgfd(ml[b], m0[b], mr[b], itermax=50, errmax=1e-10)
        assert st[b] == so == 0 and it[b] == io
        assert rel(x[b], xo) < TOL


def test_phystau_matches_oracle():
    ep = W.energy_problem(W.rel_bcc(nsets=[2] * 24), 10)
    tau = rng.normal(size=(ep.lkmax, ep.lkmax)) + 1j * rng.normal(size=(ep.lkmax, ep.lkmax))
    g = native.phystau(tau, ep.tminv[0], ep.alpha[0], ep.lmax, 1)
    o = O.phystau(tau, ep.tminv[0], ep.alpha[0], ep.lmax, 1)
    assert rel(g, o) < 1e-12


def _compare(ep, nthreads=8):
    g = api.cpacoord(ep)
    o = O.cpacoord(ep, nthreads=nthreads)
    assert o["status"] == 0 and g["status"] == 0
    assert g["cpa_iterations"] == o["cpa_iterations"]
    assert g["max_dec_iters"] == o["max_dec_iters"]
    for key in ("tauc", "taua", "taub", "tminv"):
        assert rel(g[key], o[key]) < TOL, (key, rel(g[key], o[key]))
    return g, o


@pytest.mark.parametrize("ie", [0, 7, 15])
def test_cpacoord_plain_fcc(ie):
    _compare(W.energy_problem(W.plain_fcc(nset=6), ie))


@pytest.mark.parametrize("ie", [3, 16])
def test_cpacoord_relativistic_lmax2(ie):
    spec = W.rel_bcc(nsets=[3] * 24)
    spec.lmax = 2
    _compare(W.energy_problem(spec, ie))


def test_cpacoord_relativistic_pl4_lmax3():
    spec = W.rel_bcc(nsets=[2] * 24)
    _compare(W.energy_problem(spec, 12))


def test_cpacoord_cpa_alloy_layers():
    spec = W.plain_fcc(nset=4)
    spec.alloy_layers = (1, 2, 4)
    spec.seed = 11
    g, o = _compare(W.energy_problem(spec, 6))
    assert g["cpa_iterations"] > 1


def test_cpacoord_relativistic_cpa():
    spec = W.rel_bcc_cpa(nsets=[2] * 24)
    spec.lmax = 2
    g, o = _compare(W.energy_problem(spec, 14))
    assert g["cpa_iterations"] > 1


def test_full_bz_equals_symmetrised_ibz_on_gpu():
    spec = W.plain_fcc(nset=4)
    a = api.cpacoord(W.energy_problem(spec, 4))
    b = api.cpacoord(W.energy_problem(spec, 4, kmesh="full"))
    assert rel(b["tauc"], a["tauc"]) < 1e-9


def test_decimation_divergence_is_reported_not_trapped():
    # with the 0.03 Ry j-split wells and the 2 Ry / 0.7 d_NN barrier, the
    # relativistic lmax=2 bcc stack has a k point at Im E ~ 0.07 Ry whose
    # decimation error transiently exceeds 1e10 (surfgf.f:88-93)
    spec = W.rel_bcc(nsets=[3] * 24, so_split=0.03, vscreen=2.0, rscreen=0.7)
    spec.lmax = 2
    ep = W.energy_problem(spec, 16)
    o = O.cpacoord(ep, nthreads=4)
    assert o["status"] == 2
    with pytest.raises(native.SkkrError) as ei:
        api.cpacoord(ep)
    assert ei.value.code == -4


@pytest.mark.parametrize("irel,lmax,para", [(0, 2, True), (1, 3, False)])
def test_layer_dos_kernel_matches_oracle(irel, lmax, para):
    nd = (2 if irel else 1) * (lmax + 1) ** 2
    tau = rng.normal(size=(5, nd, nd)) + 1j * rng.normal(size=(5, nd, nd))
    F = rng.normal(size=(5, nd)) + 1j * rng.normal(size=(5, nd))
    G = rng.normal(size=(5, nd)) + 1j * rng.normal(size=(5, nd))
    zm, zl = native.layer_dos(tau, F, G, lmax, irel, para)
    om, ol = O.layer_dos(tau, F, G, lmax, irel, para)
    assert rel(zm, om) < 1e-14 and rel(zl, ol) < 1e-14


def _rel_cpa_l2():
    spec = W.rel_bcc_cpa(nsets=[2] * 24)
    spec.lmax = 2
    return spec


@pytest.mark.parametrize("system,ie", [("plain", 6), ("relcpa", 14)])
def test_layer_dos_after_cpacoord(system, ie):
    """tau of cpacoord -> phystau -> layer DOS, GPU against the oracle chain."""
    from skkr_budapest_gb300 import synth as S
    spec = W.plain_fcc(nset=4) if system == "plain" else _rel_cpa_l2()
    ep = W.energy_problem(spec, ie)
    g = api.cpacoord(ep)
    o = O.cpacoord(ep, nthreads=8)
    for which in ("a", "b"):
        key = "tau" + which
        zm, zl = api.layer_dos(ep, g[key], which, para=not ep.irel)
        tinv = ep.tminva if which == "a" else ep.tminvb
        phys = np.array([O.phystau(o[key][li], tinv[li], ep.alpha[li], ep.lmax, ep.irel) for li in range(ep.nintfc)])
        F, G = S.layer_dos_inputs(ep, which)
        om, ol = O.layer_dos(phys, F, G, ep.lmax, ep.irel, not ep.irel)
        assert rel(zm, om) < TOL and rel(zl, ol) < TOL, (rel(zm, om), rel(zl, ol))


def test_cpacoord_relativistic_with_j_split():
    """The j = l +- 1/2 split well depths (0.03 Ry) on a mesh where the lead
    decimation converges: the (kappa,mu)-dependent t-matrix path."""
    spec = W.rel_bcc(nsets=[3] * 24, so_split=0.03)
    g, o = _compare(W.energy_problem(spec, 14))
    assert g["cpa_iterations"] == 1


def test_empty_k_list_is_refused_and_the_context_stays_usable():
    import dataclasses
    ep = W.energy_problem(W.plain_fcc(nset=4), 4)
    empty = dataclasses.replace(ep, xk=np.zeros((0, 2)), wk=np.zeros(0))
    ctx = api.Context.for_problem(ep)
    try:
        with pytest.raises(native.SkkrError) as ei:
            ctx.cpacoord(empty)
        assert ei.value.code == -1
        g = ctx.cpacoord(ep)
    finally:
        ctx.close()
    assert g["status"] == 0
    assert rel(g["tauc"], api.cpacoord(ep)["tauc"]) < 1e-13


def test_tau2d_export_is_the_block_tridiagonal_inverse():
    """skkr_gpu_tau2d (the Godfrin sweeps of main/tau2d.f on host arrays):
    each layer block equals the diagonal block of the inverse of the whole
    block-tridiagonal matrix with the surface operators on its corners,
    A(p,p) = M00(p), A(p,p+1) = -M01(p), A(p+1,p) = -M10(p+1),
    A(0,0) -= Y, A(last,last) -= X."""
    rng = np.random.default_rng(7)
    batch, nprc, lk, nl = 3, 3, 8, 2
    n = lk * nl

    def c(*s):
        return rng.normal(size=s) + 1j * rng.normal(size=s)

    m00 = 0.3 * c(batch, nprc, n, n) + 4 * np.eye(n)
    m01 = 0.3 * c(batch, nprc, n, n)
    m10 = 0.3 * c(batch, nprc, n, n)
    x = 0.3 * c(batch, n, n)
    y = 0.3 * c(batch, n, n)
    got = native.tau2d(m00, m01, m10, x, y, lk, wgeff=0.5)
    for k in range(batch):
        A = np.zeros((nprc * n, nprc * n), complex)
        for p in range(nprc):
            A[p * n:(p + 1) * n, p * n:(p + 1) * n] = m00[k, p]
            if p + 1 < nprc:
                A[p * n:(p + 1) * n, (p + 1) * n:(p + 2) * n] = -m01[k, p]
                A[(p + 1) * n:(p + 2) * n, p * n:(p + 1) * n] = -m10[k, p + 1]
        A[:n, :n] -= y[k]
        A[-n:, -n:] -= x[k]
        inv = np.linalg.inv(A)
        for p in range(nprc):
            for l in range(nl):
                r0 = p * n + l * lk
                ref = 0.5 * inv[r0:r0 + lk, r0:r0 + lk]
                assert np.abs(got[k, p * nl + l] - ref).max() < 1e-12 * np.abs(ref).max(), (k, p, l)
