"""Split-precision path (tcgen05 sliced products, FP32 inverse + Newton):
against numpy FP64 for the kernels and against the CPU oracle for the whole
CPA pass, at the mixed-path tolerance 1e-9 (relative Frobenius)."""
import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import api, native
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-9
rng = np.random.default_rng(5)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def crand(*s):
    return rng.normal(size=s) + 1j * rng.normal(size=s)


@pytest.mark.parametrize("n", [18, 54, 128, 256])
@pytest.mark.parametrize("slices,tol", [(5, 5e-11), (6, 3e-13), (7, 3e-14), (8, 3e-14)])
def test_sliced_zgemm_is_fp64_accurate(n, slices, tol):
    # S slices: about 2^(-8S) sigma tau per term, random-walk summed over K = 2n;
    # n <= 128 runs 8-bit digits (8 slices act as 7), n > 128 7-bit digits
    # (2^(-7S)) so that the FP32 level sums over K = 512 stay exact
    a, b = crand(3, n, n), crand(3, n, n)
    c = native.zgemm_batch(a, b, precision="mixed", slices=slices)
    ref = a @ b
    if n == 256:
        tol = {5: 2e-9, 6: 3e-11, 7: 5e-13, 8: 5e-13}[slices]  # 8: the shared tail level's floor
    for i in range(3):
        assert rel(c[i], ref[i]) < tol, rel(c[i], ref[i])


def test_sliced_zgemm_three_slices_is_fp32_class():
    n = 64
    a, b = crand(2, n, n), crand(2, n, n)
    c = native.zgemm_batch(a, b, precision="mixed", slices=3)
    e = max(rel(c[i], (a @ b)[i]) for i in range(2))
    assert 1e-12 < e < 1e-5


def test_sliced_zgemm_scaled_rows():
    # rows and columns spanning 12 orders of magnitude: per-row/column scales
    n = 40
    a = crand(2, n, n) * np.logspace(-6, 6, n)[None, :, None]
    b = crand(2, n, n) * np.logspace(4, -8, n)[None, None, :]
    c = native.zgemm_batch(a, b, precision="mixed", slices=5)
    ref = a @ b
    for i in range(2):
        err = np.abs(c[i] - ref[i]) / (np.abs(a[i]) @ np.abs(b[i]))
        assert err.max() < 5e-11


@pytest.mark.parametrize("n", [18, 54, 128])
def test_mixed_inverse_refined_to_fp64(n):
    a = crand(4, n, n) + 3 * np.eye(n)
    x, resid = native.zinv_batch(a, precision="mixed", newton=2)
    for i in range(4):
        assert rel(x[i], np.linalg.inv(a[i])) < 1e-12
    assert resid < 1e-5


@pytest.mark.parametrize("cond", [1e3, 1e5, 1e6])
def test_mixed_inverse_ill_conditioned(cond):
    # singular values spread over `cond`: the FP32 start leaves |I - AX| up
    # to ~cond 2^-24, so the larger conditions go through the further Newton
    # steps (or the FP64 redo); the result is held to FP64 accuracy
    n = 128
    u, _ = np.linalg.qr(crand(n, n))
    v, _ = np.linalg.qr(crand(n, n))
    a = np.stack([u @ np.diag(np.logspace(0, -np.log10(cond), n)) @ v.conj().T for _ in range(2)])
    a[1] = a[1].T
    x, resid = native.zinv_batch(a, precision="mixed", newton=2)
    # the floor is the residual product's rounding amplified by cond(A); two
    # plain Newton steps from the FP32 start would stop near (cond 2^-24)^4
    for i in range(2):
        ref = np.linalg.inv(a[i])
        assert rel(x[i], ref) < 2e-14 * cond, (cond, rel(x[i], ref))
        assert np.abs(a[i] @ x[i] - np.eye(n)).max() < 1e-13 * cond
    assert resid < 1e-5


def test_mixed_inverse_nan_input_is_contained():
    # a NaN item neither faults nor leaks into its batch neighbours
    n = 64
    a = crand(3, n, n) + 3 * np.eye(n)
    a[1, 5, 7] = np.nan
    x, _ = native.zinv_batch(a, precision="mixed", newton=2)
    assert np.isnan(x[1]).any()
    for i in (0, 2):
        assert rel(x[i], np.linalg.inv(a[i])) < 1e-12


def _compare_mixed(ep):
    g = api.cpacoord(ep, precision="mixed")
    o = O.cpacoord(ep, nthreads=8)
    assert o["status"] == 0 and g["status"] == 0
    assert g["cpa_iterations"] == o["cpa_iterations"]
    for key in ("tauc", "taua", "taub", "tminv"):
        assert rel(g[key], o[key]) < TOL_MIXED, (key, rel(g[key], o[key]))
    return g, o


@pytest.mark.parametrize("ie", [2, 15])
def test_mixed_cpacoord_plain_fcc(ie):
    _compare_mixed(W.energy_problem(W.plain_fcc(nset=6), ie))


def test_mixed_cpacoord_relativistic_pl4_lmax3():
    _compare_mixed(W.energy_problem(W.rel_bcc(nsets=[3] * 24), 18))


def test_mixed_cpacoord_cpa_alloy():
    spec = W.rel_bcc_cpa(nsets=[2] * 24)
    spec.lmax = 2
    g, o = _compare_mixed(W.energy_problem(spec, 14))
    assert g["cpa_iterations"] > 1


@pytest.mark.parametrize("n", [20, 54, 100])
def test_gauss_jordan_layouts_are_bit_identical(n):
    """The autotuner's thread layouts of the FP32 Gauss-Jordan give the same
    inverse bit for bit, so the choice it makes cannot change a result."""
    rng = np.random.default_rng(n)
    a = rng.normal(size=(40, n, n)) + 1j * rng.normal(size=(40, n, n)) + 3 * np.eye(n)
    outs = []
    try:
        for force in (1, 2, 3):
            native.autotune(force)
            outs.append(native.zinv_batch(a, "mixed")[0])
    finally:
        native.autotune(0)
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    tuned = native.zinv_batch(a, "mixed")[0]
    assert np.array_equal(tuned, outs[0])
    assert "n<=" in native.autotune(report=True)


@pytest.mark.parametrize("n", [65, 96, 100, 128])
def test_mixed_inverse_blocked_start_sizes(n):
    """Inverses above 64 rows start from the 2 x 2 block form (a 64-row
    leading block, the rest n - 64): refined to FP64 accuracy at every split
    (1e-11 against numpy's inverse: these random matrices reach condition
    numbers of a few hundred, and both inverses carry cond x 1e-16)."""
    a = crand(6, n, n) + 3 * np.eye(n)
    x, resid = native.zinv_batch(a, precision="mixed", newton=2)
    for i in range(6):
        assert rel(x[i], np.linalg.inv(a[i])) < 1e-11, (n, i)
    assert resid < 1e-5


def test_blocked_start_matches_whole_matrix_start():
    """The block start and the whole-matrix Gauss-Jordan start refine to the
    same k-summed tau (1e-11) on a strided sample of the benchmarked
    interface's energy 19, both within the split-precision bound of the
    oracle."""
    ep = W.energy_problem(W.rel_bcc(), 19)
    idx = np.arange(0, ep.nk, 80)
    sub = ep.with_k(ep.xk[idx], ep.wk[idx] / ep.wk[idx].sum())
    out = {}
    for blocked in (True, False):
        ctx = api.Context.for_problem(sub, "mixed")
        try:
            ctx.set_inverse_start(blocked)
            out[blocked] = ctx.cpacoord(sub)
        finally:
            ctx.close()
        assert out[blocked]["status"] == 0 and out[blocked]["max_refine_resid"] < 1e-6
    assert rel(out[True]["tauc"], out[False]["tauc"]) < 1e-11
    o = O.cpacoord(sub, nthreads=8)
    assert rel(out[True]["tauc"], o["tauc"]) < TOL_MIXED


@pytest.mark.parametrize("case", ["fcc", "rel_pl4", "rel_near_axis", "alloy"])
def test_fused_b_operand_is_bit_identical_to_staged(case):
    """The products that form their B slices in shared memory give the same
    bits as the products that load them from a staging buffer: the same
    digits in the same tile places.  Covers K = 18 (ragged k-blocks), the
    128-row interface (decimation, Newton, tau2d), an energy near the real
    axis (the exact-level tile keeps staged B for its 6-slice products) and a
    CPA alloy."""
    if case == "fcc":
        ep = W.energy_problem(W.plain_fcc(nset=6), 2)
    elif case == "alloy":
        spec = W.rel_bcc_cpa(nsets=[2] * 24)
        spec.lmax = 2
        ep = W.energy_problem(spec, 14)
    else:
        ep = W.energy_problem(W.rel_bcc(), 19 if case == "rel_pl4" else 0)
        idx = np.arange(0, ep.nk, 97)
        ep = ep.with_k(ep.xk[idx], ep.wk[idx] / ep.wk[idx].sum())
    out = {}
    for fused in (True, False):
        ctx = api.Context.for_problem(ep, "mixed")
        try:
            ctx.set_fused_split(fused)
            if case == "rel_near_axis":  # Im E = 0.016 Ry: the near-axis policy from 0.05 Ry
                ctx.set_mixed_policy(near_im=0.05)
            out[fused] = ctx.cpacoord(ep)
        finally:
            ctx.close()
        assert out[fused]["status"] == 0
    for key in ("tauc", "taua", "taub", "tminv"):
        assert np.array_equal(out[True][key], out[False][key]), key
    assert out[True]["cpa_iterations"] == out[False]["cpa_iterations"]
