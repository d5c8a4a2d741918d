"""Several systems in one call (skkr_gpu_cpacoord_many): the relativistic
PL4 lmax=3 interface, the non-relativistic PL2 lmax=2 interface and the
relativistic PL3 lmax=2 interface run concurrently (one context, stream and
host thread each) and give the results of the single calls; with kernel-class
timing on at the same time.  Several energies of one system in one call
(skkr_gpu_contour) equal their single calls."""
import numpy as np
import pytest

from skkr_budapest_gb300 import api, native
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _systems(precision_nset=3):
    return [W.energy_problem(W.rel_bcc(), 10, nset=precision_nset),
            W.energy_problem(W.nonrel_pl2(), 5, nset=precision_nset),
            W.energy_problem(W.rel_pl3_l2(), 7, nset=precision_nset)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_many_equals_single_calls(precision):
    eps = _systems()
    single = [api.cpacoord(ep, precision=precision) for ep in eps]
    native.kernel_stats_start()
    many = api.cpacoord_many(eps, precision=precision)
    ks = native.kernel_stats_stop()
    assert sum(v["launches"] for v in ks.values()) > 0
    for a, b in zip(single, many):
        assert b["status"] == 0
        assert a["cpa_iterations"] == b["cpa_iterations"]
        for key in ("tauc", "taua", "taub", "tminv"):
            assert np.array_equal(a[key], b[key]), key


def test_many_rejects_repeated_context():
    eps = _systems()[:1] * 2
    ctx = api.Context.for_problem(eps[0])
    try:
        with pytest.raises(native.SkkrError):
            api.cpacoord_many(eps, contexts=[ctx, ctx])
    finally:
        ctx.close()


def test_contour_call_equals_single_calls():
    """skkr_gpu_contour: several energies of one system in one call, each
    equal to its own skkr_gpu_cpacoord call."""
    spec = W.rel_bcc(nsets=[3] * 24)
    eps = [W.energy_problem(spec, ie) for ie in (2, 14, 20)]
    many = api.contour(eps, precision="mixed")
    for ep, r in zip(eps, many):
        one = api.cpacoord(ep, precision="mixed")
        assert r["status"] == one["status"] == 0
        assert np.array_equal(r["tauc"], one["tauc"])
