"""The library's reduction hooks on the GPU (skkr_gpu_set_reduce on host
buffers, skkr_gpu_set_reduce_device on the device buffer): two contexts,
each with half of the k points, driven by two host threads whose hook sums
the k-summed tau through a host barrier (no kernel waits on the other
context; the two only meet on the host between launches); and the device
hook through a real NCCL allreduce on a one-rank process group."""
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


def _run_split_device(ep):
    """The same two ranks through the device hook (skkr_gpu_set_reduce_device):
    each rank's hook reads the library's device buffer, the ranks meet on the
    host, and the sum is written back into that buffer before the hook
    returns (the library's stream synchronised on both sides)."""
    import torch
    bar = threading.Barrier(WORLD, timeout=120)
    bufs = [None] * WORLD
    out = [None] * WORLD

    def make_fn(rank):
        def fn(ptr, n, stream):
            torch.cuda.set_device(0)
            t = torch.as_tensor(api._DeviceDoubles(ptr, n), device="cuda")
            torch.cuda.ExternalStream(stream).synchronize()
            bufs[rank] = t.cpu()
            bar.wait()
            total = bufs[0] + bufs[1]
            bar.wait()
            t.copy_(total.cuda())
            torch.cuda.synchronize()
        return fn

    def run(rank):
        out[rank] = api.cpacoord_ksplit(ep, rank, WORLD, make_fn(rank), check=False, device_reduce=True)

    th = [threading.Thread(target=run, args=(r,)) for r in range(WORLD)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=300)
    assert all(o is not None for o in out)
    return out


def test_device_hook_contexts_equal_single_context():
    ep = _problem()
    ref = api.cpacoord(ep)
    for r in _run_split_device(ep):
        assert r["status"] == 0 and r["cpa_iterations"] == ref["cpa_iterations"]
        for key in ("tauc", "taua", "taub", "tminv"):
            assert np.linalg.norm(r[key] - ref[key]) / np.linalg.norm(ref[key]) < 1e-12, key


def test_device_hook_through_nccl():
    """torch_allreduce_device on a one-rank NCCL process group: the NCCL
    allreduce runs in place on the library's buffer, ordered on its stream."""
    import socket

    import torch.distributed as dist
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("nccl", init_method="tcp://127.0.0.1:%d" % port, rank=0, world_size=1)
    try:
        ep = _problem()
        r = api.cpacoord_ksplit(ep, 0, 1, api.torch_allreduce_device(), device_reduce=True)
    finally:
        dist.destroy_process_group()
    ref = api.cpacoord(ep)
    assert r["cpa_iterations"] == ref["cpa_iterations"]
    assert np.linalg.norm(r["tauc"] - ref["tauc"]) / np.linalg.norm(ref["tauc"]) < 1e-13
