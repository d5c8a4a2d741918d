"""Learned CPA warm start (CPU): the C4 family's inputs and targets, the
symmetry of the start, and a model file's host inference.  The ATA start has
a zero target; the free elements are those the point-group average keeps;
the start of any model is invariant under that average and equals ATA off
the alloy layers."""
import numpy as np

from skkr_budapest_gb300 import cpa_warmstart as CW


def _family():
    return CW.Family(nset=2)


def _model(tmp_path, fam, ep, scale=0.0):
    mask = CW.free_elements(ep)
    x = CW.stack_features(ep, fam)
    dims = [x.shape[1], 8, 8, 8, 2 * int(mask.sum())]
    rng = np.random.default_rng(3)
    save = {"nlayers": 4, "xmean": x.mean(0), "xstd": np.ones(x.shape[1]), "ymean": np.zeros(dims[-1]),
            "ystd": np.full(dims[-1], 1e-2), "mask": mask, "nset": fam.nset, "so_split": fam.so_split}
    for i, (a, b) in enumerate(zip(dims[:-1], dims[1:])):
        save["w%d" % i] = np.float32(rng.normal(size=(a, b)) * scale)
        save["b%d" % i] = np.zeros(b, np.float32)
    p = tmp_path / "m.npz"
    np.savez(p, **save)
    return CW.Model(str(p))


def test_features_and_targets_of_the_alloy_stack():
    fam = _family()
    rng = np.random.default_rng(0)
    ep = fam.problem(10, fam.draw(rng))
    x = CW.stack_features(ep, fam)
    assert x.shape == (4, 2 + 4 + 4 * 29)
    # the target layer comes first after E and the one-hot position
    assert np.allclose(x[:, 2:6], np.eye(4))
    assert np.allclose(x[:, 6], ep.conc[list(fam.alloy_layers)])
    mask = CW.free_elements(ep)
    assert mask.sum() == 256
    # the ATA start (what the problem carries) has a zero target
    assert np.abs(CW.stack_targets(ep, ep.tminv, fam, mask)).max() == 0.0


def test_ata_start_is_invariant_and_zero_model_gives_it(tmp_path):
    fam = _family()
    ep = fam.problem(5, fam.draw(np.random.default_rng(1)))
    P = CW.invariant_projector(ep)
    for li in fam.alloy_layers:
        assert np.abs(P(ep.tminv[li]) - ep.tminv[li]).max() < 1e-12 * np.abs(ep.tminv[li]).max()
    m0 = _model(tmp_path, fam, ep, scale=0.0)
    ws = CW.warm_start(ep, m0, fam, device="host")
    assert np.array_equal(ws, ep.tminv)


def test_start_of_a_model_is_symmetric_and_local_to_the_alloy(tmp_path):
    fam = _family()
    ep = fam.problem(7, fam.draw(np.random.default_rng(2)))
    m = _model(tmp_path, fam, ep, scale=0.3)
    ws = CW.warm_start(ep, m, fam, device="host")
    P = CW.invariant_projector(ep)
    for li in range(ep.nintfc):
        if li in fam.alloy_layers:
            assert np.all(np.isfinite(ws[li]))
            assert not np.array_equal(ws[li], ep.tminv[li])
            assert np.abs(P(ws[li]) - ws[li]).max() < 1e-10 * np.abs(ws[li]).max()
        else:
            assert np.array_equal(ws[li], ep.tminv[li])


def test_bf16_rounding_ties_to_even():
    v = np.float32([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, -2.5, 1.0 + 2.0 ** -7 + 2.0 ** -8])
    r = CW.bf16_round(v)
    assert list(r) == [1.0, np.float32(1.0 + 2.0 ** -7), -2.5, np.float32(1.0 + 2.0 ** -6)]


def test_projector_matrix_is_the_group_average_on_the_mask():
    fam = _family()
    ep = fam.problem(3, fam.draw(np.random.default_rng(4)))
    mask = CW.free_elements(ep)
    pm = CW.projector_matrix(ep, mask)
    rng = np.random.default_rng(5)
    d = np.zeros((ep.lkmax, ep.lkmax), complex)
    d[mask] = rng.normal(size=mask.sum()) + 1j * rng.normal(size=mask.sum())
    want = CW.invariant_projector(ep)(d)
    assert np.abs((pm @ d[mask]).reshape(d.shape) - want).max() < 1e-13 * np.abs(want).max()


def test_projector_cache_finds_equal_group_matrices_by_value(tmp_path):
    fam = _family()
    rng = np.random.default_rng(6)
    ep1 = fam.problem(2, fam.draw(rng))
    ep2 = fam.problem(3, fam.draw(rng))   # another energy: equal lg / rg, separate arrays
    assert ep1.lg is not ep2.lg and np.array_equal(ep1.lg, ep2.lg)
    m = _model(tmp_path, fam, ep1, scale=0.1)
    p1 = m.projector(ep1)
    p2 = m.projector(ep2)
    assert p2 is p1                       # found by value, not rebuilt
    assert m.projector(ep2) is p1         # and by identity from then on
    ep3 = fam.problem(2, fam.draw(rng))
    ep3.lg = ep3.lg * (1 + 1e-3)          # other group matrices: a new projector
    assert m.projector(ep3) is not p1
