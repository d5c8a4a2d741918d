"""ctypes front end of the CPU oracle (oracle/skkr_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The product path never imports this module.

Matrices are passed as numpy arrays of shape (..., n, n) with [row, col]
semantics; they are converted to the reference's column-major complex*16
layout at the call boundary.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in ("skkr_oracle.c", "skkr_oracle.h")):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _setup(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
D = C.c_double


class ZC(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def _zc(z):
    z = complex(z)
    return ZC(z.real, z.imag)


class G2DMap(C.Structure):
    _fields_ = [("lmax", I), ("lmmax", I), ("nslot", I), ("mi", I), ("jmax", I), ("blkmap", P),
                ("bdg", I), ("nblk", I), ("fach", ZC)]


class Problem(C.Structure):
    _fields_ = [("irel", I), ("lmax", I), ("lkmax", I), ("nprc", I), ("ninprc", P), ("bulkgeo", I),
                ("nintfc", I), ("map", P), ("nk", I), ("xk", P), ("wk", P), ("ngeff", I), ("lg", P),
                ("rg", P), ("itermaxl", I), ("itermaxr", I), ("errmax", D), ("itcpam", I),
                ("cpatol", D), ("fac", ZC), ("nblk", I), ("rstart", P), ("rvec", P), ("gR", P)]


class Result(C.Structure):
    _fields_ = [("cpa_iterations", I), ("cpa_error", D), ("sgf_status", I), ("max_dec_iters", I),
                ("dec_iters_total", C.c_int64)]


def _setup(L):
    L.orc_gjinv.argtypes = [P, I, I, P]
    L.orc_tripmt.argtypes = [P, P, P, I, I, I]
    L.orc_surfgfd.argtypes = [P, P, P, P, I, I, I, D, P]
    L.orc_surfgfd.restype = I
    L.orc_relmtrx.argtypes = [P, I, P, I, ZC, I]
    L.orc_packer.argtypes = [I, I, I, P, I, P, P, P, P, I, I, I, ZC]
    L.orc_tau2d.argtypes = [I, D, I, P, I, P, P, P, I, I, P, P, I, P, ZC]
    L.orc_dugo.argtypes = [I, P, I, P, P, I, I, P, I, P, I, I, I, ZC, I, D, P]
    L.orc_dugo.restype = I
    L.orc_tata.argtypes = [D, I, I, P, P, P]
    L.orc_phystau.argtypes = [P, P, P, P, I, I, I, I]
    L.orc_phystau2.argtypes = [P, P, P, P, P, I, I, I, I]
    L.orc_cpacoord.argtypes = [P, P, P, P, P, P, P, P, P, P, I, P, I]
    L.orc_cpacoord.restype = I
    L.orc_gk_from_rtable.argtypes = [I, P, P, P, I, D, D, P]
    L.orc_legzero.argtypes = [I, P, P]
    L.orc_zmesh_semicircle.argtypes = [I, D, D, D, P, P]
    L.orc_speck2.argtypes = [I, P, P, P, I, D, D, D, I]
    L.orc_speck2.restype = I
    L.orc_kmesh2d_ibz.argtypes = [I, I, C.c_char_p, D, D, D, P, P, P, I]
    L.orc_kmesh2d_ibz.restype = I
    L.orc_alpha_sqwell.argtypes = [ZC, D, D, I, P]
    L.orc_layer_dos.argtypes = [I, I, I, P, I, P, P, I, P, P]
    L.orc_set_reduce.argtypes = [P, P]


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def to_cm(a):
    """(..., n, n) [row, col] -> contiguous column-major complex128 buffer."""
    a = np.asarray(a, np.complex128)
    return np.array(np.swapaxes(a, -1, -2), order="C", copy=True)


def from_cm(buf):
    return np.ascontiguousarray(np.swapaxes(buf, -1, -2))


# ----------------------------------------------------------------- kernels
def gjinv(a):
    a = np.asarray(a, np.complex128)
    n = a.shape[0]
    buf = to_cm(a)
    det = np.zeros(1, np.complex128)
    lib().orc_gjinv(_ptr(buf), n, n, _ptr(det))
    return from_cm(buf), det[0]


def surfgfd(ml, m0, mr, itermax=50, errmax=1e-8):
    n = m0.shape[0]
    bl, b0, br = to_cm(ml), to_cm(m0), to_cm(mr)
    x = np.zeros_like(b0)
    it = np.zeros(1, np.int32)
    st = lib().orc_surfgfd(_ptr(bl), _ptr(b0), _ptr(br), _ptr(x), n, n, itermax, errmax, _ptr(it))
    return from_cm(x), st, int(it[0])


def relmtrx(a, fac, lmax):
    a = np.asarray(a, np.complex128)
    lm = a.shape[0]
    buf = to_cm(a)
    out = np.zeros((2 * lm, 2 * lm), np.complex128)
    lib().orc_relmtrx(_ptr(buf), lm, _ptr(out), 2 * lm, _zc(fac), lmax)
    return from_cm(out)


def tata(conc, ma, mb):
    n = ma.shape[0]
    mc = np.zeros((n, n), np.complex128)
    a, b = to_cm(ma), to_cm(mb)
    lib().orc_tata(conc, n, n, _ptr(mc), _ptr(a), _ptr(b))
    return from_cm(mc)


def phystau(tau, tinv, alpha, lmax, irel):
    n = tau.shape[0]
    t = to_cm(tau)
    ti = to_cm(tinv)
    al = np.asarray(alpha, np.complex128).copy()
    lib().orc_phystau(_ptr(t), _ptr(ti), _ptr(ti), _ptr(al), lmax, irel, n, 1)
    return from_cm(t)


def phystau2(tau, tinv1, alpha1, tinv2, alpha2, lmax, irel, idiag=0):
    """orc_phystau2: the pair block tau_ij screened -> physical with layer i's
    (tinv1, alpha1) on the rows and layer j's (tinv2, alpha2) on the columns;
    idiag=0 is the form cpacoord_ksave.f:982-988 applies to tau_ij / tau_ji."""
    n = tau.shape[0]
    t = to_cm(tau)
    t1 = to_cm(tinv1)
    t2 = to_cm(tinv2)
    a1 = np.asarray(alpha1, np.complex128).copy()
    a2 = np.asarray(alpha2, np.complex128).copy()
    lib().orc_phystau2(_ptr(t), _ptr(t1), _ptr(a1), _ptr(t2), _ptr(a2), lmax, irel, n, int(idiag))
    return from_cm(t)


def layer_dos(tau, F, G, lmax, irel, para=False):
    """orc_layer_dos: (zmom [nlay, nd], zdos_l [nlay, lmax+1]) from physical tau [nlay, nd, nd]."""
    tau = np.asarray(tau, np.complex128)
    nlay, nd = tau.shape[0], tau.shape[-1]
    t = to_cm(tau)
    f = np.ascontiguousarray(F, np.complex128).reshape(nlay, nd).copy()
    g = np.ascontiguousarray(G, np.complex128).reshape(nlay, nd).copy()
    zm = np.zeros((nlay, nd), np.complex128)
    zl = np.zeros((nlay, lmax + 1), np.complex128)
    lib().orc_layer_dos(irel, lmax, nlay, _ptr(t), nd, _ptr(f), _ptr(g), int(bool(para)), _ptr(zm), _ptr(zl))
    return zm, zl


def gk_blocks(rt, k):
    lmmax = rt.gR.shape[1]
    g = to_cm(rt.gR)
    out = np.zeros((rt.nblk, lmmax, lmmax), np.complex128)
    rs = np.ascontiguousarray(rt.rstart, np.int32)
    rv = np.ascontiguousarray(rt.rvec, np.float64)
    lib().orc_gk_from_rtable(rt.nblk, _ptr(rs), _ptr(rv), _ptr(g), lmmax, float(k[0]), float(k[1]),
                             _ptr(out))
    return from_cm(out)


def legzero(ng):
    x = np.zeros(ng)
    w = np.zeros(ng)
    lib().orc_legzero(ng, _ptr(x), _ptr(w))
    return x, w


def zmesh_semicircle(nep, eb, et, eps):
    z = np.zeros(nep, np.complex128)
    w = np.zeros(nep, np.complex128)
    lib().orc_zmesh_semicircle(nep, eb, et, eps, _ptr(z), _ptr(w))
    return z, w


def speck2(nset, ilat, alat, beta=1.0, delta=0.0, cap=200000):
    x = np.zeros(cap)
    y = np.zeros(cap)
    w = np.zeros(cap)
    nk = lib().orc_speck2(nset, _ptr(x), _ptr(y), _ptr(w), ilat, alat, beta, delta, cap)
    if nk < 0:
        raise ValueError("speck2 failed %d" % nk)
    return np.stack([x[:nk], y[:nk]], 1), w[:nk]


def kmesh2d_ibz(iset, i2dlat, idgroup, a2d, beta=1.0, delta=0.0, cap=200000):
    x = np.zeros(cap)
    y = np.zeros(cap)
    w = np.zeros(cap)
    nk = lib().orc_kmesh2d_ibz(iset, i2dlat, idgroup.encode(), a2d, beta, delta, _ptr(x), _ptr(y),
                               _ptr(w), cap)
    if nk < 0:
        raise ValueError("kmesh2d failed %d" % nk)
    return np.stack([x[:nk], y[:nk]], 1), w[:nk]


def alpha_sqwell(e, vscreen, rs, lmax):
    out = np.zeros(lmax + 1, np.complex128)
    lib().orc_alpha_sqwell(_zc(e), vscreen, rs, lmax, _ptr(out))
    return out


# ----------------------------------------------------------------- cpacoord
REDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_longlong)


def _reduce_cb(fn):
    """C callback around fn(buf: ndarray) that sums buf over ranks in place."""
    def cb(_user, buf, n):
        try:
            fn(np.ctypeslib.as_array(buf, shape=(int(n),)))
            return 0
        except Exception:  # noqa: BLE001 - reported to the C side as a failed reduction
            return 1
    return REDUCE_FN(cb)


def cpacoord(ep, nthreads=1, tminv=None, reduce=None):
    """Run the CPA + k loop of one energy problem (a workloads.EnergyProblem).
    Returns dict with tauc, taua, taub (k-summed screened, [layer,row,col]),
    tminv (converged coherent t^-1) and the loop counters.  `reduce`
    (fn(buf) summing buf over ranks in place) makes this one rank of a k-split
    energy: ep then holds this rank's k points only."""
    keep = []

    def arr(a, dt):
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a

    lk = ep.lkmax
    blk = arr(ep.blkmap, np.int32)
    bdg = ep.irel == 2
    gmap = G2DMap(ep.lmax, (ep.lmax + 1) ** 2, blk.shape[0], blk.shape[1], (blk.shape[2] - 1) // 2,
                  _ptr(blk), int(bdg), ep.rt.nblk, _zc(ep.fach if bdg else 0.0))
    nin = arr(ep.ninprc, np.int32)
    xk = arr(ep.xk, np.float64)
    wk = arr(ep.wk, np.float64)
    lg = arr(to_cm(ep.lg), np.complex128)
    rg = arr(to_cm(ep.rg), np.complex128)
    rs = arr(ep.rt.rstart, np.int32)
    rv = arr(ep.rt.rvec, np.float64)
    gR = arr(to_cm(np.concatenate([ep.rt.gR, ep.rt_h.gR]) if bdg else ep.rt.gR), np.complex128)
    pr = Problem(ep.irel, ep.lmax, lk, ep.nprc, _ptr(nin), int(ep.bulkgeo), ep.nintfc,
                 C.cast(C.pointer(gmap), C.c_void_p), len(xk), _ptr(xk), _ptr(wk), len(lg), _ptr(lg),
                 _ptr(rg), ep.itermaxl, ep.itermaxr, ep.errmax, ep.itcpam, ep.cpatol, _zc(ep.fac),
                 ep.rt.nblk, _ptr(rs), _ptr(rv), _ptr(gR))
    conc = arr(ep.conc, np.float64)
    tl = arr(to_cm(ep.tminvl), np.complex128)
    tr = arr(to_cm(ep.tminvr), np.complex128)
    ti = arr(to_cm(ep.tminv if tminv is None else tminv), np.complex128).copy()
    ta = arr(to_cm(ep.tminva), np.complex128)
    tb = arr(to_cm(ep.tminvb), np.complex128)
    n = ep.nintfc
    tauc = np.zeros((n, lk, lk), np.complex128)
    taua = np.zeros_like(tauc)
    taub = np.zeros_like(tauc)
    res = Result()
    cb = _reduce_cb(reduce) if reduce is not None else None
    if cb is not None:
        lib().orc_set_reduce(C.cast(cb, C.c_void_p), None)
    try:
        st = lib().orc_cpacoord(C.cast(C.pointer(pr), C.c_void_p), _ptr(conc), _ptr(tl), _ptr(tr),
                                _ptr(ti), _ptr(ta), _ptr(tb), _ptr(tauc), _ptr(taua), _ptr(taub), lk,
                                C.cast(C.pointer(res), C.c_void_p), nthreads)
    finally:
        if cb is not None:
            lib().orc_set_reduce(None, None)
    return dict(status=st, tauc=from_cm(tauc), taua=from_cm(taua), taub=from_cm(taub),
                tminv=from_cm(ti), cpa_iterations=res.cpa_iterations, cpa_error=res.cpa_error,
                sgf_status=res.sgf_status, max_dec_iters=res.max_dec_iters,
                dec_iters_total=res.dec_iters_total)


def tauij(ep, pairs, a1, a2, cvec, a0mat, tminv=None, nthreads=1):
    """Off-diagonal k sums of one energy problem with fixed t^-1 (no CPA
    update): for each pair (n1, n2, li, lj) the inter-site tau between layer
    li in cell 0 and layer lj in cell n1 a1 + n2 a2, and back
    (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:760-840 with tau2d_god.f);
    a0mat[g] is the 2x2 in-plane rotation of group operation g, cvec[l] the
    in-plane position of interface layer l.  Returns dict tau_ij, tau_ji
    [pair,row,col], tauc [layer,row,col], status."""
    keep = []

    def arr(a, dt):
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a

    lk = ep.lkmax
    blk = arr(ep.blkmap, np.int32)
    bdg = ep.irel == 2
    gmap = G2DMap(ep.lmax, (ep.lmax + 1) ** 2, blk.shape[0], blk.shape[1], (blk.shape[2] - 1) // 2,
                  _ptr(blk), int(bdg), ep.rt.nblk, _zc(ep.fach if bdg else 0.0))
    nin = arr(ep.ninprc, np.int32)
    xk = arr(ep.xk, np.float64)
    wk = arr(ep.wk, np.float64)
    lg = arr(to_cm(ep.lg), np.complex128)
    rg = arr(to_cm(ep.rg), np.complex128)
    rs = arr(ep.rt.rstart, np.int32)
    rv = arr(ep.rt.rvec, np.float64)
    gR = arr(to_cm(np.concatenate([ep.rt.gR, ep.rt_h.gR]) if bdg else ep.rt.gR), np.complex128)
    pr = Problem(ep.irel, ep.lmax, lk, ep.nprc, _ptr(nin), int(ep.bulkgeo), ep.nintfc,
                 C.cast(C.pointer(gmap), C.c_void_p), len(xk), _ptr(xk), _ptr(wk), len(lg), _ptr(lg),
                 _ptr(rg), ep.itermaxl, ep.itermaxr, ep.errmax, ep.itcpam, ep.cpatol, _zc(ep.fac),
                 ep.rt.nblk, _ptr(rs), _ptr(rv), _ptr(gR))
    tl = arr(to_cm(ep.tminvl), np.complex128)
    tr = arr(to_cm(ep.tminvr), np.complex128)
    ti = arr(to_cm(ep.tminv if tminv is None else tminv), np.complex128)
    pa = arr(np.asarray(pairs, np.int32).reshape(-1, 4), np.int32)
    npair = len(pa)
    va1 = arr(a1, np.float64)
    va2 = arr(a2, np.float64)
    cv = arr(np.asarray(cvec, np.float64).reshape(-1, 2), np.float64)
    am = arr(np.asarray(a0mat, np.float64).reshape(-1, 4), np.float64)
    tij = np.zeros((max(npair, 1), lk, lk), np.complex128)
    tji = np.zeros_like(tij)
    tauc = np.zeros((ep.nintfc, lk, lk), np.complex128)
    L = lib()
    L.orc_tauij.restype = C.c_int
    st = L.orc_tauij(C.cast(C.pointer(pr), C.c_void_p), _ptr(tl), _ptr(tr), _ptr(ti), npair, _ptr(pa),
                     _ptr(va1), _ptr(va2), _ptr(cv), _ptr(am), _ptr(tij), _ptr(tji), _ptr(tauc), lk,
                     nthreads)
    return dict(status=st, tau_ij=from_cm(tij)[:npair], tau_ji=from_cm(tji)[:npair], tauc=from_cm(tauc))


def tau2dgod_k(ep, ik, tminv=None):
    """Full layer-pair tau of one k point (ngeff classes ignored: the first
    group element only), for checks against a direct inverse."""
    ep1 = ep.with_k(ep.xk[ik:ik + 1], np.array([1.0]))
    ep1.lg, ep1.rg = ep.lg[:1], ep.rg[:1]
    n = ep.nintfc
    pairs = [(0, 0, a, b) for a in range(n) for b in range(n)]
    r = tauij(ep1, pairs, [1.0, 0.0], [0.0, 1.0], np.zeros((n, 2)), [[1.0, 0.0, 0.0, 1.0]], tminv=tminv)
    return r["tau_ij"].reshape(n, n, ep.lkmax, ep.lkmax)
