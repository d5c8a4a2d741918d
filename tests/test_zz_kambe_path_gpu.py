"""The path on the reference's own k-space structure constants
(skkr_gpu_stage_kambe: Kambe lattice sums per distinct layer separation,
slab screening G (1 - alpha G)^-1 by the batched Gauss-Jordan kernel, the
central blocks into the structure-constant cache) against the oracle's
k loop run one k point at a time on the blocks of its gstore + scrstr
restatement (oracle/kambe.py), with barriers that localise the screened
constants: non-relativistic fcc(001) lmax=2 and the relativistic bcc(001)
PL4 lmax=3 interface of the benchmarked workload.  The slab of 28 layers
(N = 448, the size of the reference's C2 screening slab) runs through the
same path."""
import dataclasses

import numpy as np
import pytest

import kambe as K
import oracle as O
from skkr_budapest_gb300 import api, kspace
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _oracle_tau(ep, form):
    """The oracle's k loop per k point on a table holding that k's blocks of
    the reference's G(k) (one entry per block at R = 0)."""
    st = form
    lat = K.Lattice2D([np.sqrt(st["area"]), 0.0], [0.0, np.sqrt(st["area"])])
    tau = 0
    for ik in range(ep.nk):
        rt = ep.rt
        blocks = K.slab_table_blocks(st["e"], ep.xk[ik][0], ep.xk[ik][1], ep.lmax, st["pos"], list(st["alpha"]), lat,
                                     rt.blk_of_j, st["centre"])
        fake = S.RTable(rt.lmax, rt.nblk, np.arange(rt.nblk + 1, dtype=np.int32), np.zeros((rt.nblk, 2)),
                        np.ascontiguousarray(blocks), rt.jmax, rt.blk_of_j)
        r = O.cpacoord(dataclasses.replace(ep, xk=ep.xk[ik:ik + 1], wk=ep.wk[ik:ik + 1], rt=fake), nthreads=8)
        assert r["status"] == 0
        tau = tau + r["tauc"]
    return tau


def _run(ep, form, precision="fp64"):
    ctx = api.Context.for_problem(ep, precision)
    try:
        return ctx.cpacoord_kambe(ep, form)
    finally:
        ctx.close()


def test_nonrelativistic_path_on_the_kambe_form():
    spec = W.plain_fcc(nset=4)
    spec.vscreen, spec.rscreen = 4.0, 0.5
    ep = W.energy_problem(spec, 8)
    form = kspace.kambe_form(ep, spec, nl=8)
    g = _run(ep, form)
    ref = _oracle_tau(ep, form)
    assert g["status"] == 0
    assert np.linalg.norm(g["tauc"] - ref) / np.linalg.norm(ref) < 1e-9


def test_relativistic_interface_on_the_kambe_form():
    spec = W.rel_bcc()
    ep = W.energy_problem(spec, 12)
    ep = ep.with_k(ep.xk[::90], ep.wk[::90] / ep.wk[::90].sum())
    form = kspace.kambe_form(ep, spec, nl=10)
    g = _run(ep, form)
    ref = _oracle_tau(ep, form)
    assert g["status"] == 0
    assert np.linalg.norm(g["tauc"] - ref) / np.linalg.norm(ref) < 1e-9
    # the split-precision path on the same G(k)
    m = _run(ep, form, "mixed")
    assert np.linalg.norm(m["tauc"] - ref) / np.linalg.norm(ref) < 1e-9


def test_slab_of_the_reference_size():
    # 28 layers x 16 = 448: the screening slab of the reference's C2 interface
    spec = W.rel_bcc()
    ep = W.energy_problem(spec, 12)
    ep = ep.with_k(ep.xk[:3], ep.wk[:3] / ep.wk[:3].sum())
    big = _run(ep, kspace.kambe_form(ep, spec, nl=28))
    small = _run(ep, kspace.kambe_form(ep, spec, nl=20))
    assert big["status"] == small["status"] == 0
    # the slab converges with thickness under the sample's screening
    assert np.linalg.norm(big["tauc"] - small["tauc"]) / np.linalg.norm(big["tauc"]) < 1e-6
