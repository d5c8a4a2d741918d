"""Host tau files (.tau): the physical tau of the layered host that the
cluster-embedding code reads.

After its CPA loop, the cpacoord of the BdG layer code
(skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:949-1036) turns the k-summed pair
blocks tau_ij, tau_ji (phystau2, idiag = 0) and the layer-diagonal coherent
tau (phystau) into the physical representation, and its root rank writes them
with tauhout (skkr_dbogo_bsf/clu/tauhout.f:2-102; the relativistic layer
code's cluster/rsp-lay/tauhout.f has the same records).  The cluster code
reads them back with tauhin (skkr_dbogo_bsf/clu/tauhin.f:2-165).

One file per energy, named taupath + ie in four digits + '.tau'
(`write(temp,'(i4.4)') ie`), Fortran unformatted sequential, each record
framed by its byte length as a 4-byte little-endian integer before and after:

    [ie int32] [ce complex*16] [nk int32] [npair int32]
    per pair q = 1..npair:  [q int32] [kpair(1:4) int32] [tau_ij n*n] [tau_ji n*n]
    per layer l = 1..nintfc: [l int32] [tau_ii n*n]

with every matrix complex*16 in column-major order and n the basis size.
kpair = (n1, n2, li, lj): the second site sits in the cell
R = n1 a1 + n2 a2 of layer lj, the first in cell 0 of layer li; the file holds
1-based layers, the arrays of this package 0-based ones, and the functions
below convert.

`read_tauh` keeps tauhin's rules: the stored energy must equal the one asked
for to 1e-15, and a requested pair is found either as stored or as the
reversed pair (-n1, -n2, lj, li), whose tau_ij and tau_ji then trade places.
It reads every stored pair record before the layer records (tauhin skips the
pair records when no pair is requested, which would misread a file that has
some), and a requested pair that is not in the file is an error, as the
'pair mismatch' stop of tauhin."""
from __future__ import annotations

import os
import struct

import numpy as np

ENERGY_TOL = 1.0e-15   # skkr_dbogo_bsf/clu/tauhin.f: 'data tol/1.0d-15/'


class TauhError(RuntimeError):
    pass


def tauh_path(taupath, ie) -> str:
    """taupath // ie as four digits // '.tau' (tauhout.f, tauhin.f)."""
    ie = int(ie)
    if not 0 <= ie <= 9999:
        raise ValueError("energy index %d does not fit the four-digit file name" % ie)
    return os.fspath(taupath) + "%04d.tau" % ie


def _put(f, payload: bytes):
    n = len(payload)
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def _get(f) -> bytes:
    head = f.read(4)
    if len(head) < 4:
        raise TauhError("end of file")
    (n,) = struct.unpack("<i", head)
    payload = f.read(n)
    tail = f.read(4)
    if len(payload) != n or len(tail) != 4 or struct.unpack("<i", tail)[0] != n:
        raise TauhError("corrupt record (length markers disagree)")
    return payload


def _ints(rec, count, what):
    if len(rec) != 4 * count:
        raise TauhError("%s: record of %d bytes, expected %d" % (what, len(rec), 4 * count))
    return struct.unpack("<%di" % count, rec)


def _mat(rec, n, what):
    if len(rec) != 16 * n * n:
        raise TauhError("%s: record of %d bytes for n = %d" % (what, len(rec), n))
    return np.frombuffer(rec, np.complex128).reshape((n, n), order="F")


def _file_pair(p):
    n1, n2, li, lj = (int(v) for v in p)
    return (n1, n2, li + 1, lj + 1)


def write_tauh(taupath, ie, ce, nk, pairs, tau_ij, tau_ji, tau_ii) -> str:
    """tauhout: write one energy's physical tau.  pairs (npair, 4) as
    (n1, n2, li, lj) with 0-based layers; tau_ij, tau_ji (npair, n, n);
    tau_ii (nintfc, n, n).  Returns the file name."""
    pairs = np.asarray(pairs, np.int64).reshape(-1, 4)
    tau_ij = np.asarray(tau_ij, np.complex128)
    tau_ji = np.asarray(tau_ji, np.complex128)
    tau_ii = np.asarray(tau_ii, np.complex128)
    npair = len(pairs)
    n = tau_ii.shape[-1]
    if tau_ii.ndim != 3 or tau_ii.shape[1] != n:
        raise ValueError("tau_ii must be (nintfc, n, n)")
    if npair and (tau_ij.shape != (npair, n, n) or tau_ji.shape != (npair, n, n)):
        raise ValueError("tau_ij and tau_ji must be (npair, n, n) with the basis size of tau_ii")
    for p in pairs:
        if not (0 <= p[2] < len(tau_ii) and 0 <= p[3] < len(tau_ii)):
            raise ValueError("pair %s names a layer outside 0..%d" % (tuple(p), len(tau_ii) - 1))
    path = tauh_path(taupath, ie)
    with open(path, "wb") as f:
        _put(f, struct.pack("<i", int(ie)))
        _put(f, np.array([complex(ce)], np.complex128).tobytes())
        _put(f, struct.pack("<i", int(nk)))
        _put(f, struct.pack("<i", npair))
        for q in range(npair):
            _put(f, struct.pack("<i", q + 1))
            _put(f, struct.pack("<4i", *_file_pair(pairs[q])))
            # ((tau(k1,k2),k1=1,n),k2=1,n): column-major
            _put(f, tau_ij[q].tobytes(order="F"))
            _put(f, tau_ji[q].tobytes(order="F"))
        for li in range(len(tau_ii)):
            _put(f, struct.pack("<i", li + 1))
            _put(f, tau_ii[li].tobytes(order="F"))
    return path


def read_tauh(taupath, ie, ze, pairs, nintfc, n) -> dict:
    """tauhin: read one energy's physical tau for the requested pairs
    ((n1, n2, li, lj), 0-based layers).  Returns ie, ce, nk and the arrays
    tau_ij, tau_ji (npair, n, n), tau_ii (nintfc, n, n)."""
    pairs = [tuple(int(v) for v in p) for p in np.asarray(pairs, np.int64).reshape(-1, 4)]
    with open(tauh_path(taupath, ie), "rb") as f:
        (ieread,) = _ints(_get(f), 1, "energy index")
        rec = _get(f)
        if len(rec) != 16:
            raise TauhError("energy record of %d bytes" % len(rec))
        ce = complex(np.frombuffer(rec, np.complex128)[0])
        (nk,) = _ints(_get(f), 1, "number of k points")
        (npairin,) = _ints(_get(f), 1, "number of pairs")
        if abs(complex(ze) - ce) > ENERGY_TOL:
            raise TauhError("energy mismatch: file %s has %r, asked for %r" % (tauh_path(taupath, ie), ce, complex(ze)))
        stored = {}
        for q in range(npairin):
            _ints(_get(f), 1, "pair index")
            kp = _ints(_get(f), 4, "pair")
            tij = _mat(_get(f), n, "tau_ij of pair %d" % (q + 1))
            tji = _mat(_get(f), n, "tau_ji of pair %d" % (q + 1))
            stored.setdefault(kp, (tij, tji))
        tau_ij = np.zeros((len(pairs), n, n), np.complex128)
        tau_ji = np.zeros_like(tau_ij)
        for q, p in enumerate(pairs):
            n1, n2, li, lj = _file_pair(p)
            if (n1, n2, li, lj) in stored:
                tau_ij[q], tau_ji[q] = stored[(n1, n2, li, lj)]
            elif (-n1, -n2, lj, li) in stored:
                tau_ji[q], tau_ij[q] = stored[(-n1, -n2, lj, li)]
            else:
                raise TauhError("pair mismatch: %s is not in the file, directly or reversed" % (p,))
        tau_ii = np.zeros((int(nintfc), n, n), np.complex128)
        for li in range(int(nintfc)):
            (lab,) = _ints(_get(f), 1, "layer index")
            if lab != li + 1:
                raise TauhError("layer record %d labelled %d" % (li + 1, lab))
            tau_ii[li] = _mat(_get(f), n, "tau_ii of layer %d" % (li + 1))
    return dict(ie=ieread, ce=ce, nk=nk, tau_ij=tau_ij, tau_ji=tau_ji, tau_ii=tau_ii)
