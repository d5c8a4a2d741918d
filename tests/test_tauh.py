"""Host tau files (.tau, skkr_dbogo_bsf/clu/tauhout.f and tauhin.f): byte
layout of the Fortran unformatted records, round trips with pairs asked for
directly and reversed, tauhin's energy and pair checks, and the screened ->
physical transform of the pair blocks (phystau2.f) in the oracle against its
closed form (CPU)."""
import struct

import numpy as np
import pytest

import oracle as O
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import tauh
from skkr_budapest_gb300 import workloads as W

rng = np.random.default_rng(5)


def crand(*s):
    return rng.normal(size=s) + 1j * rng.normal(size=s)


def rec(payload):
    return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))


def test_record_layout(tmp_path):
    # n = 1, one pair (1, -1, layer 0 -> layer 1), two layers
    ce = 0.5 + 0.01j
    tij = np.array([[[1 + 2j]]])
    tji = np.array([[[3 + 4j]]])
    tii = np.array([[[5 + 6j]], [[7 + 8j]]])
    path = tauh.write_tauh(str(tmp_path / "host"), 12, ce, 300, [(1, -1, 0, 1)], tij, tji, tii)
    assert path.endswith("host0012.tau")
    z = lambda v: np.array([v], np.complex128).tobytes()
    expect = (rec(struct.pack("<i", 12)) + rec(z(ce)) + rec(struct.pack("<i", 300)) + rec(struct.pack("<i", 1)) +
              rec(struct.pack("<i", 1)) + rec(struct.pack("<4i", 1, -1, 1, 2)) + rec(z(1 + 2j)) + rec(z(3 + 4j)) +
              rec(struct.pack("<i", 1)) + rec(z(5 + 6j)) + rec(struct.pack("<i", 2)) + rec(z(7 + 8j)))
    assert open(path, "rb").read() == expect


def test_matrices_are_column_major(tmp_path):
    t = np.array([[[1, 2], [3, 4]]], np.complex128)      # t[0] = [[1, 2], [3, 4]] (row, col)
    path = tauh.write_tauh(str(tmp_path / "h"), 1, 0.1j, 1, [], np.zeros((0, 2, 2)), np.zeros((0, 2, 2)), t)
    raw = open(path, "rb").read()
    body = raw[-(64 + 4):-4]                              # the last record's payload
    assert np.array_equal(np.frombuffer(body, np.complex128), [1, 3, 2, 4])


def test_round_trip_direct_and_reversed(tmp_path):
    n, nl = 9, 6
    pairs = [(0, 0, 0, 1), (1, 0, 0, 0), (1, 1, 2, 3), (0, -1, 3, 1)]
    tij, tji, tii = crand(4, n, n), crand(4, n, n), crand(nl, n, n)
    ce = 0.3 + 0.02j
    tauh.write_tauh(str(tmp_path / "h"), 7, ce, 4321, pairs, tij, tji, tii)
    # ask in another order, two of them reversed: (-n1, -n2, lj, li)
    want = [(1, 1, 2, 3), (0, 0, 1, 0), (-1, 0, 0, 0), (0, 1, 1, 3)]
    r = tauh.read_tauh(str(tmp_path / "h"), 7, ce, want, nl, n)
    assert r["ie"] == 7 and r["nk"] == 4321 and r["ce"] == ce
    assert np.array_equal(r["tau_ii"], tii)
    assert np.array_equal(r["tau_ij"][0], tij[2]) and np.array_equal(r["tau_ji"][0], tji[2])
    assert np.array_equal(r["tau_ij"][1], tji[0]) and np.array_equal(r["tau_ji"][1], tij[0])
    # (1, 0, 0, 0) reversed is (-1, 0, 0, 0): same layers, opposite cell
    assert np.array_equal(r["tau_ij"][2], tji[1]) and np.array_equal(r["tau_ji"][2], tij[1])
    assert np.array_equal(r["tau_ij"][3], tji[3]) and np.array_equal(r["tau_ji"][3], tij[3])


def test_reader_checks(tmp_path):
    n = 2
    tauh.write_tauh(str(tmp_path / "h"), 3, 0.2 + 0.1j, 10, [(0, 0, 0, 1)], crand(1, n, n), crand(1, n, n),
                    crand(2, n, n))
    with pytest.raises(tauh.TauhError, match="energy mismatch"):
        tauh.read_tauh(str(tmp_path / "h"), 3, 0.2 + 0.1j + 1e-13, [(0, 0, 0, 1)], 2, n)
    with pytest.raises(tauh.TauhError, match="pair mismatch"):
        tauh.read_tauh(str(tmp_path / "h"), 3, 0.2 + 0.1j, [(1, 0, 0, 1)], 2, n)
    with pytest.raises(tauh.TauhError):
        tauh.read_tauh(str(tmp_path / "h"), 3, 0.2 + 0.1j, [(0, 0, 0, 1)], 2, n + 1)   # wrong basis size
    with pytest.raises(tauh.TauhError, match="end of file"):
        tauh.read_tauh(str(tmp_path / "h"), 3, 0.2 + 0.1j, [(0, 0, 0, 1)], 3, n)       # one layer too many
    # no pair asked for: the stored pair records are still read past
    r = tauh.read_tauh(str(tmp_path / "h"), 3, 0.2 + 0.1j, [], 2, n)
    assert r["tau_ij"].shape == (0, n, n) and r["tau_ii"].shape == (2, n, n)


def test_writer_checks(tmp_path):
    with pytest.raises(ValueError):
        tauh.tauh_path(str(tmp_path / "h"), 10000)
    with pytest.raises(ValueError):
        tauh.write_tauh(str(tmp_path / "h"), 1, 0.1j, 1, [(0, 0, 0, 2)], crand(1, 2, 2), crand(1, 2, 2),
                        crand(2, 2, 2))


def _lof(irel, lmax):
    if irel == 0:
        return [l for l in range(lmax + 1) for _ in range(2 * l + 1)]
    lm = (lmax + 1) ** 2
    lof, l = [], 0
    while len(lof) < 2 * lm:
        lof += [l] * (2 if l == 0 else 4 * l + 2)
        l += 1
    lof = lof[:2 * lm]
    return lof + [x + lmax + 1 for x in lof] if irel == 2 else lof


@pytest.mark.parametrize("irel,lmax", [(0, 2), (1, 3), (2, 1)])
def test_oracle_phystau2_closed_form(irel, lmax):
    # (1 + A1 t1) tau (1 + t2 A2) [- (A1 + A1 t1 A2)], A = diag(alpha[l(index)])
    lm = (lmax + 1) ** 2
    nd = lm if irel == 0 else 2 * lm if irel == 1 else 4 * lm
    nal = lmax + 1 if irel < 2 else 2 * (lmax + 1)
    tau, t1, t2 = crand(nd, nd), crand(nd, nd), crand(nd, nd)
    a1, a2 = crand(nal), crand(nal)
    lof = _lof(irel, lmax)
    A1, A2 = np.diag(a1[lof]), np.diag(a2[lof])
    want = (np.eye(nd) + A1 @ t1) @ tau @ (np.eye(nd) + t2 @ A2)
    got = O.phystau2(tau, t1, a1, t2, a2, lmax, irel)
    assert np.abs(got - want).max() < 1e-14 * np.abs(want).max()
    got1 = O.phystau2(tau, t1, a1, t2, a2, lmax, irel, idiag=1)
    want1 = want - (A1 + A1 @ t1 @ A2)
    assert np.abs(got1 - want1).max() < 1e-14 * np.abs(want1).max()
    # one layer on both sides: phystau
    assert np.allclose(O.phystau(tau, t1, a1, lmax, irel), O.phystau2(tau, t1, a1, t1, a1, lmax, irel, 1),
                       rtol=0, atol=1e-15 * np.abs(want).max())


def test_oracle_host_tau_file(tmp_path):
    # the oracle's pair sums and CPA tau through phystau2 / phystau into a file
    # and back: what the cluster code would read for this interface
    spec, ie = W.plain_fcc(nset=4), 4
    ep = W.energy_problem(spec, ie)
    a2d = spec.stacking.a2d
    l0, n = int(ep.ninprc[0]), ep.nintfc
    cvec = np.array([[0.5 * ((l0 + l) % 2) * a2d] * 2 for l in range(n)])
    pairs = [(0, 0, 0, 1), (1, 0, 0, 0), (1, 1, 2, 3)]
    a0mat = [o[:2, :2].T.ravel() for o in S.c4v_ops()]
    c = O.cpacoord(ep, nthreads=4)
    o = O.tauij(ep, pairs, [a2d, 0.0], [0.0, a2d], cvec, a0mat, tminv=c["tminv"], nthreads=4)
    tminv, al = c["tminv"], ep.alpha
    tij = np.array([O.phystau2(o["tau_ij"][q], tminv[i], al[i], tminv[j], al[j], ep.lmax, ep.irel)
                    for q, (_, _, i, j) in enumerate(pairs)])
    tji = np.array([O.phystau2(o["tau_ji"][q], tminv[j], al[j], tminv[i], al[i], ep.lmax, ep.irel)
                    for q, (_, _, i, j) in enumerate(pairs)])
    tii = np.array([O.phystau(c["tauc"][l], tminv[l], al[l], ep.lmax, ep.irel) for l in range(n)])
    tauh.write_tauh(str(tmp_path / "host"), ie + 1, ep.ce, ep.nk, pairs, tij, tji, tii)
    r = tauh.read_tauh(str(tmp_path / "host"), ie + 1, ep.ce, [(0, 0, 1, 0)], n, ep.lkmax)
    assert np.array_equal(r["tau_ij"][0], tji[0]) and np.array_equal(r["tau_ii"], tii)
