"""The library's reduction hook (skkr_gpu_set_reduce) on the GPU: two
contexts, each with half of the k points, driven by two host threads whose
hook sums the k-summed tau through a host barrier (no kernel waits on the
other context; the two only meet on the host between launches)."""
import threading

import numpy as np
import pytest

from skkr_budapest_gb300 import api
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu
WORLD = 2


def _problem():
    spec = W.plain_fcc(nset=4)
    spec.alloy_layers = (2, 3)
    return W.energy_problem(spec, 6)


def _run_split(ep, fail_rank=-1):
    bar = threading.Barrier(WORLD, timeout=120)
    bufs = [None] * WORLD
    out = [None] * WORLD

    def make_fn(rank):
        def fn(buf):
            bufs[rank] = buf.copy()
            bar.wait()
            total = bufs[0] + bufs[1]
            bar.wait()
            buf[:] = total
        return fn

    def run(rank):
        e = ep
        if rank == fail_rank:
            import copy
            e = copy.copy(ep)
            e.itermaxl = e.itermaxr = 1
        out[rank] = api.cpacoord_ksplit(e, rank, WORLD, make_fn(rank), check=False)

    th = [threading.Thread(target=run, args=(r,)) for r in range(WORLD)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=300)
    assert all(o is not None for o in out)
    return out


def test_ksplit_contexts_equal_single_context():
    ep = _problem()
    ref = api.cpacoord(ep)
    assert ref["cpa_iterations"] > 1
    res = _run_split(ep)
    for r in res:
        assert r["status"] == 0
        assert r["cpa_iterations"] == ref["cpa_iterations"]
        for key in ("tauc", "taua", "taub", "tminv"):
            err = np.linalg.norm(r[key] - ref[key]) / np.linalg.norm(ref[key])
            assert err < 1e-12, (key, err)


def test_ksplit_failed_rank_reports_to_peer():
    res = _run_split(_problem(), fail_rank=1)
    assert res[1]["status"] == -3      # SKKR_ERR_SGF_ITERMAX on the failing rank
    assert res[0]["status"] == -8      # SKKR_ERR_PEER on the other
