"""The decimation loop as one CUDA graph launch per k chunk (a WHILE node
whose iteration count, convergence test and further Newton steps of the
split-precision inverse are decided on the device) against the same loop
driven from the host one iteration at a time: identical results and
iteration counts on the FP64 and the split-precision path."""
import numpy as np
import pytest

from skkr_budapest_gb300 import api
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _both(ep, precision):
    out = []
    for graphs in (False, True):
        ctx = api.Context.for_problem(ep, precision)
        try:
            ctx.set_graphs(graphs)
            out.append(ctx.cpacoord(ep))
        finally:
            ctx.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_decimation_equals_host_loop(precision):
    ep = W.energy_problem(W.rel_bcc(nsets=[4] * 24), 19)
    host, graph = _both(ep, precision)
    assert host["status"] == graph["status"] == 0
    assert host["max_dec_iters"] == graph["max_dec_iters"]
    assert host["dec_iters_total"] == graph["dec_iters_total"]
    for key in ("tauc", "taua", "taub"):
        assert np.array_equal(host[key], graph[key]), key
    if precision == "mixed":
        assert host["inv_refined"] == graph["inv_refined"]
        assert host["max_refine_resid"] == graph["max_refine_resid"]


def test_graph_decimation_with_alloy_layers_and_near_axis():
    # CPA iterations after the first reuse the cached surface operators; the
    # energy nearest the axis runs the 7-slice exact-level products
    spec = W.rel_bcc_cpa(nsets=[2] * 24)
    spec.lmax = 2
    for ie in (14, 23):
        host, graph = _both(W.energy_problem(spec, ie), "mixed")
        assert host["cpa_iterations"] == graph["cpa_iterations"]
        assert np.array_equal(host["tauc"], graph["tauc"])
        assert np.array_equal(host["tminv"], graph["tminv"])
