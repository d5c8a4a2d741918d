"""Effective t-matrix files (.tcpa, main/tcpaio.f): byte layout of the
Fortran unformatted records, round trips over several energies, the energy
check of tcpa_in, and the warm start they exist for: a CPA loop started from
the stored converged matrices needs a single update (oracle, CPU)."""
import struct

import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import tcpa
from skkr_budapest_gb300 import workloads as W

rng = np.random.default_rng(11)


def crand(*s):
    return rng.normal(size=s) + 1j * rng.normal(size=s)


def test_record_layout(tmp_path):
    # one energy, one alloy layer of n = 2, one pure layer (c = 1): the file is
    # [16][ce][16] [64][t(1,1) t(2,1) t(1,2) t(2,2)][64]
    p = tmp_path / "t.tcpa"
    ce = 0.25 + 0.125j
    t = np.array([[[1 + 2j, 3 + 4j], [5 + 6j, 7 + 8j]], [[9, 9], [9, 9]]], np.complex128)
    with tcpa.TcpaWriter(p) as w:
        w.write(ce, [0.5, 1.0], t)
    raw = p.read_bytes()
    expect = (struct.pack("<i", 16) + np.array([ce]).tobytes() + struct.pack("<i", 16) +
              struct.pack("<i", 64) + np.array([1 + 2j, 5 + 6j, 3 + 4j, 7 + 8j]).tobytes() +
              struct.pack("<i", 64))
    assert raw == expect


def test_round_trip_over_energies(tmp_path):
    p = tmp_path / "t.tcpa"
    n, nl = 8, 5
    conc = [0.3, 1.0, 0.9, 1.0 - 1e-7, 0.5]       # layers 2 and 4 are not alloys
    energies = [0.1 + 0.2j, 0.3 + 0.1j, 0.5 + 0.01j]
    mats = [crand(nl, n, n) for _ in energies]
    with tcpa.TcpaWriter(p) as w:
        for ce, m in zip(energies, mats):
            w.write(ce, conc, m)
    with tcpa.TcpaReader(p) as r:
        for ce, m in zip(energies, mats):
            out = np.full((nl, n, n), 7.0 + 0j)
            r.read(ce, conc, out)
            for li in range(nl):
                if 1.0 - conc[li] > tcpa.TINY:
                    assert np.array_equal(out[li], m[li])
                else:
                    assert np.all(out[li] == 7.0)      # untouched, as tcpa_in
        with pytest.raises(tcpa.TcpaError):
            r.read(energies[0], conc, np.zeros((nl, n, n), np.complex128))   # end of file


def test_energy_check(tmp_path):
    p = tmp_path / "t.tcpa"
    with tcpa.TcpaWriter(p) as w:
        w.write(0.5 + 0.1j, [0.5], crand(1, 4, 4))
    with tcpa.TcpaReader(p) as r:
        with pytest.raises(tcpa.TcpaError, match="check energy array"):
            r.read(0.5 + 0.1j + 1e-9, [0.5], np.zeros((1, 4, 4), np.complex128))


def test_truncated_file(tmp_path):
    p = tmp_path / "t.tcpa"
    with tcpa.TcpaWriter(p) as w:
        w.write(0.5 + 0.1j, [0.5], crand(1, 4, 4))
    p.write_bytes(p.read_bytes()[:-10])
    with tcpa.TcpaReader(p) as r:
        with pytest.raises(tcpa.TcpaError):
            r.read(0.5 + 0.1j, [0.5], np.zeros((1, 4, 4), np.complex128))


def test_warm_start_from_stored_matrices(tmp_path):
    # the reference's use: converged m_c of one run written with tcpa_out, read
    # back with tcpa_in as the start of the next run of the same energy
    spec = W.rel_bcc_cpa(nsets=[1] * 24)
    spec.lmax = 1
    ep = W.energy_problem(spec, 14)
    first = O.cpacoord(ep, nthreads=4)
    assert first["status"] == 0 and first["cpa_iterations"] > 2
    conc = np.asarray(ep.conc)
    p = tmp_path / "run.tcpa"
    with tcpa.TcpaWriter(p) as w:
        w.write(ep.ce, conc, first["tminv"])
    start = np.array(ep.tminv, np.complex128, copy=True)
    with tcpa.TcpaReader(p) as r:
        r.read(ep.ce, conc, start)
    again = O.cpacoord(ep, nthreads=4, tminv=start)
    assert again["status"] == 0
    assert again["cpa_iterations"] <= 2
    rel = np.linalg.norm(again["tauc"] - first["tauc"]) / np.linalg.norm(first["tauc"])
    assert rel < 1e-9
