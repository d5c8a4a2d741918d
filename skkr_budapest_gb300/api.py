"""Host-side mirror of the reference's cpacoord interface over the C ABI.

`cpacoord(ep)` has the argument meaning of the Fortran routine
(skkr_kpar_v6/rsp-scf/cpacoord_ksave.f:3-9): complex energy, k points and
weights, point-group matrices, lead / interface / species inverse t-matrices
and concentrations in; k-summed coherent tau, species tau and the converged
coherent t^-1 out.  Like the Fortran it fails loudly: a decimation that does
not converge raises (the reference `stop`s, main/surfgf.f:98-101).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N


class Context:
    """Device context for one system (sizes fixed, energies vary)."""

    def __init__(self, irel, lmax, nprc, ninprc, ngeff, itermaxl=50, itermaxr=50, errmax=1e-8,
                 itcpam=50, cpatol=1e-10, precision="fp64", nk_chunk=0, slices=0):
        s = N.Sizes()
        s.mode = N.REL if irel else N.NONREL
        s.lmax = lmax
        s.nprc = nprc
        for i, v in enumerate(ninprc):
            s.ninprc[i] = int(v)
        s.bulkgeo = 1
        s.ngeff = ngeff
        s.itermaxl, s.itermaxr, s.errmax = itermaxl, itermaxr, errmax
        s.itcpam, s.cpatol = itcpam, cpatol
        s.precision = {"fp64": N.FP64, "mixed": N.MIXED}[precision]
        s.nk_chunk = nk_chunk
        s.slices = slices
        self.sizes = s
        self.lk = 2 * (lmax + 1) ** 2 if irel else (lmax + 1) ** 2
        self.nintfc = int(sum(ninprc[1:nprc + 1]))
        h = C.c_void_p()
        rc = N.lib().skkr_gpu_create(C.cast(C.pointer(s), C.c_void_p), C.cast(C.pointer(h), C.c_void_p))
        N._check(rc, "skkr_gpu_create")
        self.h = h
        self._keep = None

    @classmethod
    def for_problem(cls, ep, precision="fp64", nk_chunk=0, slices=0):
        return cls(ep.irel, ep.lmax, ep.nprc, ep.ninprc, len(ep.lg), ep.itermaxl, ep.itermaxr, ep.errmax,
                   ep.itcpam, ep.cpatol, precision, nk_chunk, slices)

    def close(self):
        if self.h:
            N.lib().skkr_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- split form -------------------------------------------------------
    def _host_inputs(self, ep, tminv=None):
        rt = N.RTableHolder(ep.rt, ep.blkmap)
        arrs = dict(
            xk=np.ascontiguousarray(ep.xk, np.float64), wk=np.ascontiguousarray(ep.wk, np.float64),
            lg=N.cm(ep.lg), rg=N.cm(ep.rg), conc=np.ascontiguousarray(ep.conc, np.float64),
            tl=N.cm(ep.tminvl), tr=N.cm(ep.tminvr),
            ti=N.cm(ep.tminv if tminv is None else tminv), ta=N.cm(ep.tminva), tb=N.cm(ep.tminvb))
        return rt, arrs

    def stage(self, ep, tminv=None):
        rt, a = self._host_inputs(ep, tminv)
        self._keep = (rt, a)
        p = N._p
        rc = N.lib().skkr_gpu_stage(self.h, ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag, rt.ptr(),
                                    len(a["xk"]), p(a["xk"]), p(a["wk"]), p(a["lg"]), p(a["rg"]),
                                    p(a["conc"]), p(a["tl"]), p(a["tr"]), p(a["ti"]), p(a["ta"]),
                                    p(a["tb"]), self.lk)
        N._check(rc, "skkr_gpu_stage")

    def run(self, check=True):
        st = N.Status()
        rc = N.lib().skkr_gpu_run(self.h, C.cast(C.pointer(st), C.c_void_p))
        if check:
            N._check(rc, "skkr_gpu_run")
        return st

    def fetch(self):
        n, lk = self.nintfc, self.lk
        out = {k: np.zeros((n, lk, lk), np.complex128) for k in ("tminv", "tauc", "taua", "taub")}
        p = N._p
        rc = N.lib().skkr_gpu_fetch(self.h, p(out["tminv"]), p(out["tauc"]), p(out["taua"]), p(out["taub"]),
                                    lk)
        N._check(rc, "skkr_gpu_fetch")
        return {k: N.uncm(v) for k, v in out.items()}

    # -- several energies resident at once -----------------------------------
    def stage_slot(self, slot, ep, tminv=None):
        rt, a = self._host_inputs(ep, tminv)
        if not hasattr(self, "_slot_keep"):
            self._slot_keep = {}
        self._slot_keep[slot] = (rt, a)
        p = N._p
        rc = N.lib().skkr_gpu_stage_slot(self.h, slot, ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag,
                                         rt.ptr(), len(a["xk"]), p(a["xk"]), p(a["wk"]), p(a["lg"]),
                                         p(a["rg"]), p(a["conc"]), p(a["tl"]), p(a["tr"]), p(a["ti"]),
                                         p(a["ta"]), p(a["tb"]), self.lk)
        N._check(rc, "skkr_gpu_stage_slot")

    def run_slot(self, slot, check=True):
        st = N.Status()
        rc = N.lib().skkr_gpu_run_slot(self.h, slot, C.cast(C.pointer(st), C.c_void_p))
        if check:
            N._check(rc, "skkr_gpu_run_slot")
        return st

    def fetch_slot(self, slot):
        n, lk = self.nintfc, self.lk
        out = {k: np.zeros((n, lk, lk), np.complex128) for k in ("tminv", "tauc", "taua", "taub")}
        p = N._p
        rc = N.lib().skkr_gpu_fetch_slot(self.h, slot, p(out["tminv"]), p(out["tauc"]), p(out["taua"]),
                                         p(out["taub"]), lk)
        N._check(rc, "skkr_gpu_fetch_slot")
        return {k: N.uncm(v) for k, v in out.items()}

    # -- one call, host buffers in and out (the drop-in form) ---------------
    def cpacoord(self, ep, tminv=None, check=True):
        rt, a = self._host_inputs(ep, tminv)
        n, lk = self.nintfc, self.lk
        out = {k: np.zeros((n, lk, lk), np.complex128) for k in ("tauc", "taua", "taub")}
        st = N.Status()
        p = N._p
        rc = N.lib().skkr_gpu_cpacoord(self.h, ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag,
                                       rt.ptr(), len(a["xk"]), p(a["xk"]), p(a["wk"]), p(a["lg"]),
                                       p(a["rg"]), p(a["conc"]), p(a["tl"]), p(a["tr"]), p(a["ti"]),
                                       p(a["ta"]), p(a["tb"]), p(out["tauc"]), p(out["taua"]),
                                       p(out["taub"]), lk, C.cast(C.pointer(st), C.c_void_p))
        if check:
            N._check(rc, "skkr_gpu_cpacoord")
        res = {k: N.uncm(v) for k, v in out.items()}
        res["tminv"] = N.uncm(a["ti"])
        res.update(status=rc, cpa_iterations=st.cpa_iterations, cpa_error=st.cpa_error,
                   max_dec_iters=st.max_dec_iters, dec_iters_total=st.dec_iters_total,
                   gpu_launches=st.gpu_launches, ik=st.ik, run_ms=st.run_ms,
                   h2d_bytes=sum(v.nbytes for v in a.values()) + rt.gR.nbytes + rt.rvec.nbytes,
                   d2h_bytes=sum(v.nbytes for v in out.values()))
        return res


def cpacoord(ep, precision="fp64", tminv=None, check=True, slices=0):
    """One energy through the GPU path (creates a context for the call)."""
    ctx = Context.for_problem(ep, precision, slices=slices)
    try:
        return ctx.cpacoord(ep, tminv=tminv, check=check)
    finally:
        ctx.close()
