"""Effective t-matrix files (.tcpa): the reference's CPA warm-start store.

The reference writes, after every energy's CPA loop, the converged inverse
effective t-matrices of the alloy layers to unit 10 (main/tcpaio.f:251-276,
called from rsp-scf/skkr.f:450) and reads them back as the starting point of
the CPA loop from the `laymat` / `leftmat` / `rightmat` files
(main/tcpaio.f:193-249, rsp-scf/skkr.f:395).  The files are Fortran
unformatted sequential (`form='unformatted'`, main/tcpaio.f:163-170): per
energy one record holding the complex*16 energy, then one record per layer
whose concentration leaves an alloy (1 - c > 1e-6) holding its n x n
complex*16 matrix in column-major order.  Each record is framed by its byte
length as a 4-byte integer before and after (the gfortran and ifort default
record markers), little-endian on both the x86 and Arm hosts.

`TcpaWriter` / `TcpaReader` mirror tcpa_out / tcpa_in: energies follow one
another in the order the caller writes them; the reader checks each record's
energy against the one it is asked for (|ce - cein| <= 1e-12, where the
reference stops with 'check energy array') and leaves the non-alloy layers
untouched.  The arrays are numpy (nlayers, n, n) complex128, the layout the
rest of this package uses; `n` is the basis size (2 (lmax+1)^2 for the
relativistic code)."""
from __future__ import annotations

import struct

import numpy as np

TINY = 1.0e-6          # main/tcpaio.f: 'data tiny/1.0d-6/'
ENERGY_TOL = 1.0e-12   # main/tcpaio.f:219,229,239


class TcpaError(RuntimeError):
    pass


def _alloy(conc):
    return [1.0 - float(c) > TINY for c in conc]


def _put(f, payload: bytes):
    n = len(payload)
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def _get(f) -> bytes:
    head = f.read(4)
    if len(head) < 4:
        raise TcpaError("end of file")
    (n,) = struct.unpack("<i", head)
    payload = f.read(n)
    tail = f.read(4)
    if len(payload) != n or len(tail) != 4 or struct.unpack("<i", tail)[0] != n:
        raise TcpaError("corrupt record (length markers disagree)")
    return payload


class TcpaWriter:
    """tcpa_out: append one energy's alloy-layer matrices per call."""

    def __init__(self, path):
        self.f = open(path, "wb")

    def write(self, ce, conc, tminv):
        tminv = np.asarray(tminv, np.complex128)
        if tminv.ndim != 3 or tminv.shape[1] != tminv.shape[2] or len(conc) != tminv.shape[0]:
            raise ValueError("tminv must be (nlayers, n, n) with one concentration per layer")
        _put(self.f, np.array([complex(ce)], np.complex128).tobytes())
        for li, cpalay in enumerate(_alloy(conc)):
            if cpalay:
                # column-major, as the Fortran implied do ((t(k1,k2),k1=1,n),k2=1,n)
                _put(self.f, np.asfortranarray(tminv[li]).tobytes(order="F"))

    def close(self):
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class TcpaReader:
    """tcpa_in: read the next energy's alloy-layer matrices into `tminv`."""

    def __init__(self, path):
        self.f = open(path, "rb")

    def read(self, ce, conc, tminv):
        tminv = np.asarray(tminv)
        n = tminv.shape[1]
        rec = _get(self.f)
        if len(rec) != 16:
            raise TcpaError("energy record of %d bytes" % len(rec))
        cein = np.frombuffer(rec, np.complex128)[0]
        if abs(complex(ce) - cein) > ENERGY_TOL:
            raise TcpaError("check energy array: file has %r, asked for %r" % (cein, complex(ce)))
        for li, cpalay in enumerate(_alloy(conc)):
            if cpalay:
                rec = _get(self.f)
                if len(rec) != 16 * n * n:
                    raise TcpaError("layer %d: record of %d bytes for n = %d" % (li + 1, len(rec), n))
                tminv[li] = np.frombuffer(rec, np.complex128).reshape((n, n), order="F")
        return tminv

    def close(self):
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
