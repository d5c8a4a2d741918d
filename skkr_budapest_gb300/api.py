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
        s.mode = {0: N.NONREL, 1: N.REL, 2: N.BDG}[int(irel)]
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
        self.lk = (4 if irel == 2 else 2 if irel else 1) * (lmax + 1) ** 2
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

    def set_mixed_policy(self, dec_fp64_im=2e-4, near_im=1e-3, slices_near=7, dominant_frac=1e-2):
        """Precision near the real axis (skkr_gpu_set_mixed_policy): FP64
        decimation below |Im E| = dec_fp64_im, slices_near BF16 slices for the
        products below |Im E| = near_im, FP64 redo of every k point carrying
        more than dominant_frac of the k-summed tau."""
        N._check(N.lib().skkr_gpu_set_mixed_policy(self.h, dec_fp64_im, near_im, slices_near, dominant_frac),
                 "skkr_gpu_set_mixed_policy")

    def set_newton(self, steps=2):
        """Standard Newton steps of the split-precision inverse (skkr_gpu_set_newton)."""
        N._check(N.lib().skkr_gpu_set_newton(self.h, int(steps)), "skkr_gpu_set_newton")

    def set_inverse_start(self, blocked=True):
        """FP32 start of split-precision inverses above 64 rows: 2 x 2 blocks
        (default) or the whole-matrix Gauss-Jordan (skkr_gpu_set_inverse_start)."""
        N._check(N.lib().skkr_gpu_set_inverse_start(self.h, 1 if blocked else 0), "skkr_gpu_set_inverse_start")

    def set_fused_split(self, on=True):
        """B operands of the split-precision products formed inside the
        product (default) or split into staging buffers first; the same
        result bit for bit (skkr_gpu_set_fused_split)."""
        N._check(N.lib().skkr_gpu_set_fused_split(self.h, 1 if on else 0), "skkr_gpu_set_fused_split")

    def set_graphs(self, on=True):
        """Decimation loop as one CUDA graph launch per k chunk (the default)
        or one host-driven iteration at a time (skkr_gpu_set_graphs)."""
        N._check(N.lib().skkr_gpu_set_graphs(self.h, 1 if on else 0), "skkr_gpu_set_graphs")

    def set_reduce(self, fn):
        """Make this context one rank of a k-split energy: fn(buf) must sum
        the float64 host buffer over the ranks in place (an allreduce) and is
        called once per CPA iteration (skkr_gpu_set_reduce).  None clears it."""
        self._reduce_cb = N.reduce_callback(fn) if fn is not None else None
        N._check(N.lib().skkr_gpu_set_reduce(self.h, C.cast(self._reduce_cb, C.c_void_p) if fn else None, None),
                 "skkr_gpu_set_reduce")

    def set_reduce_device(self, fn):
        """The same with the sum done on the device (skkr_gpu_set_reduce_device):
        fn(ptr, n, stream) must sum the n doubles at device address ptr over
        the ranks in place, ordered on the CUDA stream `stream`."""
        self._reduce_dev_cb = N.reduce_device_callback(fn) if fn is not None else None
        N._check(N.lib().skkr_gpu_set_reduce_device(self.h, C.cast(self._reduce_dev_cb, C.c_void_p) if fn else None,
                                                    None), "skkr_gpu_set_reduce_device")

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
        rt = N.RTableHolder(ep.rt, ep.blkmap, hole=ep.rt_h if ep.irel == 2 else None)
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

    def cpacoord_kambe(self, ep, form, tminv=None, check=True):
        """One energy with the reference's k-space G_scr(k) (the Kambe sums and
        slab screening of kspace.kambe_form) in place of the table transform:
        stage, skkr_gpu_stage_kambe, run, fetch."""
        self.stage(ep, tminv)
        al = np.ascontiguousarray(form["alpha"], np.complex128)
        keep = (form["pos"], al, form["gvec"], form["rvec"])
        kf = N.KambeForm(form["e"].real, form["e"].imag, int(form["nl"]), N._p(keep[0]), N._p(al),
                         int(form["centre"]), N._p(keep[2]), len(keep[2]), N._p(keep[3]), len(keep[3]),
                         float(form["area"]), float(form["factor"]), float(form["gcut"]), float(form["rcut"]))
        N._check(N.lib().skkr_gpu_stage_kambe(self.h, C.cast(C.pointer(kf), C.c_void_p)), "skkr_gpu_stage_kambe")
        st = self.run(check=check)
        out = self.fetch() if st.code == 0 else {}
        out.update(status=st.code, cpa_iterations=st.cpa_iterations, max_dec_iters=st.max_dec_iters,
                   run_ms=st.run_ms, gpu_launches=st.gpu_launches)
        return out

    def tauij(self, ep, pairs, a1, a2, cvec, a0mat, tminv=None, check=True):
        """Off-diagonal tau of the interface for cluster embedding
        (skkr_gpu_tauij): stages ep (with tminv as the coherent t^-1) and
        runs one k loop; pairs are (n1, n2, li, lj), 0-based layers.  Returns
        tau_ij, tau_ji as (npair, lk, lk) arrays and the status."""
        self.stage(ep, tminv)
        pa = np.ascontiguousarray(np.asarray(pairs, np.int32).reshape(-1, 4))
        npair, lk = len(pa), self.lk
        va1 = np.ascontiguousarray(a1, np.float64)
        va2 = np.ascontiguousarray(a2, np.float64)
        cv = np.ascontiguousarray(np.asarray(cvec, np.float64).reshape(-1, 2))
        am = np.ascontiguousarray(np.asarray(a0mat, np.float64).reshape(-1, 4))
        oij = np.zeros((npair, lk, lk), np.complex128)
        oji = np.zeros_like(oij)
        st = N.Status()
        p = N._p
        rc = N.lib().skkr_gpu_tauij(self.h, npair, p(pa), p(va1), p(va2), p(cv), p(am), p(oij), p(oji), lk,
                                    C.cast(C.pointer(st), C.c_void_p))
        if check:
            N._check(rc, "skkr_gpu_tauij")
        return dict(status=rc, tau_ij=N.uncm(oij), tau_ji=N.uncm(oji), gpu_launches=st.gpu_launches,
                    max_dec_iters=st.max_dec_iters)

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
        """One energy through the reference-facing call skkr_gpu_cpacoord
        (BdG: skkr_gpu_cpacoord_bdg) with host buffers in and out."""
        rt, a = self._host_inputs(ep, tminv)
        n, lk = self.nintfc, self.lk
        out = {k: np.zeros((n, lk, lk), np.complex128) for k in ("tauc", "taua", "taub")}
        st = N.Status()
        p = N._p
        tail = (rt.ptr(), len(a["xk"]), p(a["xk"]), p(a["wk"]), p(a["lg"]), p(a["rg"]), p(a["conc"]),
                p(a["tl"]), p(a["tr"]), p(a["ti"]), p(a["ta"]), p(a["tb"]), p(out["tauc"]), p(out["taua"]),
                p(out["taub"]), lk, C.cast(C.pointer(st), C.c_void_p))
        if ep.irel == 2:
            fach = complex(ep.fach)
            rc = N.lib().skkr_gpu_cpacoord_bdg(self.h, ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag,
                                               fach.real, fach.imag, *tail)
        else:
            rc = N.lib().skkr_gpu_cpacoord(self.h, ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag, *tail)
        if check:
            N._check(rc, "skkr_gpu_cpacoord")
        res = {k: N.uncm(v) for k, v in out.items()}
        res["tminv"] = N.uncm(a["ti"])
        res.update(status=rc, cpa_iterations=st.cpa_iterations, cpa_error=st.cpa_error,
                   max_dec_iters=st.max_dec_iters, dec_iters_total=st.dec_iters_total,
                   gpu_launches=st.gpu_launches, ik=st.ik, run_ms=st.run_ms,
                   max_refine_resid=st.max_refine_resid, inv_fallbacks=st.inv_fallbacks, k_fp64=st.k_fp64,
                   inv_refined=st.inv_refined, alg_flops=st.alg_flops,
                   h2d_bytes=sum(v.nbytes for v in a.values()) + rt.gR.nbytes + rt.rvec.nbytes,
                   d2h_bytes=sum(v.nbytes for v in out.values()))
        return res


def ksplit_indices(nk, rank, world):
    """k points of `rank` in the round-robin split of cpacoord_ksave.f:189
    (modulo(ik-1, nprocs) == myrank)."""
    return np.arange(rank, nk, world)


def ksplit_problem(ep, rank, world):
    """The EnergyProblem of one rank of a k-split energy: its own k points
    with their global weights (the k-sum is completed by the allreduce)."""
    idx = ksplit_indices(ep.nk, rank, world)
    if len(idx) == 0:
        raise ValueError("rank %d of %d has no k points (nk=%d)" % (rank, world, ep.nk))
    return ep.with_k(ep.xk[idx], ep.wk[idx])


def torch_allreduce(group=None):
    """fn(buf) that sums a float64 host buffer over the ranks of a
    torch.distributed group in place: gloo on the host tensor, NCCL through a
    device copy."""
    import torch
    import torch.distributed as dist

    def fn(buf):
        t = torch.from_numpy(buf)
        if dist.get_backend(group) == "nccl":
            d = t.to("cuda")
            dist.all_reduce(d, group=group)
            t.copy_(d.cpu())
        else:
            dist.all_reduce(t, group=group)
    return fn


class _DeviceDoubles:
    """A view of n doubles at a device address, for torch.as_tensor."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 2}


def torch_allreduce_device(group=None):
    """fn(ptr, n, stream) for Context.set_reduce_device: an in-place
    torch.distributed allreduce (NCCL) of the library's device buffer,
    ordered on the library's stream (no host copy)."""
    import torch
    import torch.distributed as dist

    def fn(ptr, n, stream):
        t = torch.as_tensor(_DeviceDoubles(ptr, n), device="cuda")
        s = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            dist.all_reduce(t, group=group)
    return fn


def cpacoord_ksplit(ep, rank, world, allreduce, precision="fp64", slices=0, check=True, device_reduce=False):
    """One rank of an energy whose k points are split over `world` ranks:
    the library runs this rank's k points and calls `allreduce` on the
    k-summed tau before every CPA update, so every rank returns the full
    result.  device_reduce: `allreduce` is a device hook (fn(ptr, n, stream),
    e.g. torch_allreduce_device) instead of a host one."""
    epl = ksplit_problem(ep, rank, world)
    ctx = Context.for_problem(epl, precision, slices=slices)
    try:
        if device_reduce:
            ctx.set_reduce_device(allreduce)
        else:
            ctx.set_reduce(allreduce)
        return ctx.cpacoord(epl, check=check)
    finally:
        ctx.close()


def cpacoord_many(eps, precision="fp64", check=True, slices=0, contexts=None):
    """One energy of each of several systems in one call
    (skkr_gpu_cpacoord_many): every system has its own context, stream and
    host thread inside the library.  Returns the list of per-system results
    of `Context.cpacoord`."""
    own = contexts is None
    ctxs = [Context.for_problem(ep, precision, slices=slices) for ep in eps] if own else list(contexts)
    try:
        keep, outs, args = [], [], (N.EnergyArgs * len(eps))()
        p = N._p
        for i, (ctx, ep) in enumerate(zip(ctxs, eps)):
            rt, a = ctx._host_inputs(ep, None)
            n, lk = ctx.nintfc, ctx.lk
            out = {k: np.zeros((n, lk, lk), np.complex128) for k in ("tauc", "taua", "taub")}
            keep.append((rt, a))
            outs.append(out)
            fach = complex(ep.fach) if ep.irel == 2 else 0j
            args[i] = N.EnergyArgs(ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag, fach.real, fach.imag,
                                   rt.ptr(), len(a["xk"]), p(a["xk"]), p(a["wk"]), p(a["lg"]), p(a["rg"]),
                                   p(a["conc"]), p(a["tl"]), p(a["tr"]), p(a["ti"]), p(a["ta"]), p(a["tb"]),
                                   p(out["tauc"]), p(out["taua"]), p(out["taub"]), lk)
        hs = (C.c_void_p * len(eps))(*[c.h.value for c in ctxs])
        sts = (N.Status * len(eps))()
        rc = N.lib().skkr_gpu_cpacoord_many(len(eps), C.cast(hs, C.c_void_p), C.cast(args, C.c_void_p),
                                           C.cast(sts, C.c_void_p))
        if check:
            N._check(rc, "skkr_gpu_cpacoord_many")
        res = []
        for (rt, a), out, st in zip(keep, outs, sts):
            r = {k: N.uncm(v) for k, v in out.items()}
            r["tminv"] = N.uncm(a["ti"])
            r.update(status=st.code, cpa_iterations=st.cpa_iterations, cpa_error=st.cpa_error,
                     max_dec_iters=st.max_dec_iters, dec_iters_total=st.dec_iters_total,
                     gpu_launches=st.gpu_launches, run_ms=st.run_ms, alg_flops=st.alg_flops)
            res.append(r)
        return res
    finally:
        if own:
            for c in ctxs:
                c.close()


def contour(eps, precision="fp64", check=True, slices=0, context=None):
    """Several energies of one system in one call (skkr_gpu_contour), in
    order on one context.  Returns the per-energy results of
    Context.cpacoord."""
    own = context is None
    ctx = Context.for_problem(eps[0], precision, slices=slices) if own else context
    try:
        keep, outs, args = [], [], (N.EnergyArgs * len(eps))()
        p = N._p
        for i, ep in enumerate(eps):
            rt, a = ctx._host_inputs(ep, None)
            n, lk = ctx.nintfc, ctx.lk
            out = {k: np.zeros((n, lk, lk), np.complex128) for k in ("tauc", "taua", "taub")}
            keep.append((rt, a))
            outs.append(out)
            fach = complex(ep.fach) if ep.irel == 2 else 0j
            args[i] = N.EnergyArgs(ep.ce.real, ep.ce.imag, ep.fac.real, ep.fac.imag, fach.real, fach.imag,
                                   rt.ptr(), len(a["xk"]), p(a["xk"]), p(a["wk"]), p(a["lg"]), p(a["rg"]),
                                   p(a["conc"]), p(a["tl"]), p(a["tr"]), p(a["ti"]), p(a["ta"]), p(a["tb"]),
                                   p(out["tauc"]), p(out["taua"]), p(out["taub"]), lk)
        sts = (N.Status * len(eps))()
        rc = N.lib().skkr_gpu_contour(ctx.h, len(eps), C.cast(args, C.c_void_p), C.cast(sts, C.c_void_p))
        if check:
            N._check(rc, "skkr_gpu_contour")
        res = []
        for (rt, a), out, st in zip(keep, outs, sts):
            r = {k: N.uncm(v) for k, v in out.items()}
            r["tminv"] = N.uncm(a["ti"])
            r.update(status=st.code, cpa_iterations=st.cpa_iterations, cpa_error=st.cpa_error,
                     max_dec_iters=st.max_dec_iters, dec_iters_total=st.dec_iters_total,
                     gpu_launches=st.gpu_launches, run_ms=st.run_ms, alg_flops=st.alg_flops)
            res.append(r)
        return res
    finally:
        if own:
            ctx.close()


def cpacoord(ep, precision="fp64", tminv=None, check=True, slices=0):
    """One energy through the GPU path (creates a context for the call)."""
    ctx = Context.for_problem(ep, precision, slices=slices)
    try:
        return ctx.cpacoord(ep, tminv=tminv, check=check)
    finally:
        ctx.close()


BSF_NAMES = ("bsfe", "bsfh", "bsfeh", "bsfhe", "bsfteh", "bsfthe")


def bsf(ep, kpts, cpa=None, para=False, precision="fp64"):
    """Bloch spectral function of the interface layers at the k points kpts
    ((nk, 2), a.u.), CPA and BdG forms included, as the BdG code's spectral
    mode does (skkr_dbogo_bsf/rsp-scf/skkr.f:688-712 and 1076-1090: the
    converged CPA of the energy is read back by tcpa_in, cpacoord runs per k
    point without CPA iterations, then bsf.f).  `cpa` is the result of
    Context.cpacoord for ep over its own k mesh (run here when None): its
    coherent t^-1 m_c and k-integrated tau_c, tau_A, tau_B.  Each k point is a
    one-point k loop with the identity alone on m_c for every layer (no alloy,
    so no CPA iteration); every tau goes through phystau on the device
    (tau_c, tau(k) with m_c; tau_A, tau_B with their species' t^-1); then
    skkr_gpu_bsf with the radial overlaps of the model's wells
    (synth.bsf_radial) and, for BdG, the pairing operators
    (synth.pairing_kmy).  Returns {name: [nk, nintfc]} for bsfe and, for BdG,
    bsfh, bsfeh, bsfhe, bsfteh, bsfthe (bsf.f's output names)."""
    import dataclasses
    from . import synth as S
    if cpa is None:
        cpa = cpacoord(ep, precision)
    mc = np.asarray(cpa["tminv"])
    layers = range(ep.nintfc)

    def phys(tau, tinv):
        return np.array([N.phystau(tau[li], tinv[li], ep.alpha[li], ep.lmax, ep.irel) for li in layers])

    tc = phys(cpa["tauc"], mc)
    ta = phys(cpa["taua"], ep.tminva)
    tb = phys(cpa["taub"], ep.tminvb)
    one = dataclasses.replace(ep, lg=ep.lg[:1], rg=ep.rg[:1], conc=np.ones(ep.nintfc), tminv=mc.copy(),
                              tminva=mc.copy(), tminvb=mc.copy())
    kpts = np.asarray(kpts, float).reshape(-1, 2)
    nd = ep.lkmax
    tk = np.zeros((len(kpts), ep.nintfc, nd, nd), complex)
    ctx = Context.for_problem(one, precision)
    try:
        for i, k in enumerate(kpts):
            r = ctx.cpacoord(one.with_k(k[None, :], np.ones(1)))
            tk[i] = phys(r["tauc"], mc)
    finally:
        ctx.close()
    F, Feh = S.bsf_radial(ep)
    pair = None
    if ep.irel == 2:
        P = S.pairing_kmy(ep.lmax)
        pair = np.array([P[name] for name in ("singlet", "t0", "tup", "tdown")])
    out = N.bsf(ep.irel, ep.lmax, ep.conc, tk, tc, ta, tb, F, Feh, pair, para)
    names = BSF_NAMES if ep.irel == 2 else BSF_NAMES[:1]
    return {name: out[:, :, i] for i, name in enumerate(names)}


def layer_dos(ep, tau, which="a", para=False):
    """Layer DOS of the interface layers of one energy, as locquant.f does
    after cpacoord: screened -> physical tau (phystau) per layer, then
    zmom_i = -1/pi (F_i tau_ii - G_i) and its sums per orbital l, both on the
    device.  `tau` is the k-summed screened tau of species `which` (taua or
    taub of cpacoord); F, G are the square-well radial integrals of that
    species.  Returns (zmom [nintfc, lk], zdos_l [nintfc, lmax+1]); the DOS is
    the imaginary part."""
    from . import synth as S
    tinv = ep.tminva if which == "a" else ep.tminvb
    phys = np.array([N.phystau(tau[li], tinv[li], ep.alpha[li], ep.lmax, ep.irel) for li in range(ep.nintfc)])
    F, G = S.layer_dos_inputs(ep, which)
    return N.layer_dos(phys, F, G, ep.lmax, ep.irel, para)


def host_tau(ep, tminv, tauc, tij, pairs):
    """The physical tau that the BdG layer code hands to the cluster code
    (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:976-1016), on the device: every
    pair block of `tij` (Context.tauij: k-summed, screened) through phystau2
    with layer li's screening on the rows and layer lj's on the columns
    (tau_ji the other way round, idiag = 0), every layer of the k-summed
    coherent `tauc` (Context.cpacoord) through phystau.  `tminv` is the
    coherent t^-1 both were computed with; pairs are (n1, n2, li, lj),
    0-based layers.  Returns tau_ij, tau_ji (npair, lk, lk), tau_ii
    (nintfc, lk, lk)."""
    pa = np.asarray(pairs, np.int64).reshape(-1, 4)
    lmax, irel, al = ep.lmax, ep.irel, ep.alpha
    tau_ij = np.array([N.phystau2(tij["tau_ij"][q], tminv[li], al[li], tminv[lj], al[lj], lmax, irel)
                       for q, (_, _, li, lj) in enumerate(pa)]).reshape(len(pa), ep.lkmax, ep.lkmax)
    tau_ji = np.array([N.phystau2(tij["tau_ji"][q], tminv[lj], al[lj], tminv[li], al[li], lmax, irel)
                       for q, (_, _, li, lj) in enumerate(pa)]).reshape(len(pa), ep.lkmax, ep.lkmax)
    tau_ii = np.array([N.phystau(tauc[li], tminv[li], al[li], lmax, irel) for li in range(ep.nintfc)])
    return dict(tau_ij=tau_ij, tau_ji=tau_ji, tau_ii=tau_ii)


def write_host_tau(taupath, ie, ep, tminv, tauc, tij, pairs):
    """tauhout after cpacoord: host_tau, then the .tau file of energy index ie
    (the reference's 1-based contour index, part of the file name) with the
    number of k points of ep.  Returns the file name."""
    from . import tauh
    h = host_tau(ep, tminv, tauc, tij, pairs)
    return tauh.write_tauh(taupath, ie, ep.ce, ep.nk, pairs, h["tau_ij"], h["tau_ji"], h["tau_ii"])


def bloch_spectral(ep, kpts, which="a", para=False):
    """Bloch spectral function of the interface layers at the k points kpts
    ((nk, 2), a.u.), for layers without an alloy (rsp-scf/bsf.f with the
    coherent tau of those layers, skkr_dbogo_bsf/rsp-scf/bsf.f:236-240):
        A_l(k, E) = -1/pi Im sum_{L in l} F_L tau_LL(k),
    tau(k) the physical site-diagonal tau of that one k point (no point-group
    average), F the single-site radial integrals of the layer DOS; the
    k-independent single-site term of the DOS is not part of it.  Each k
    point is a one-point k loop of cpacoord with the identity alone, then
    phystau and the layer-DOS kernel with G = 0, all on the device.  Returns
    (A_l [nk, nintfc, lmax+1], A_L [nk, nintfc, lk]).  Alloy layers need
    the CPA form of bsf.f (its A0 and A1 terms): `bsf` below."""
    import dataclasses
    from . import synth as S
    if any(1e-6 < c < 1 - 1e-6 for c in ep.conc):
        raise ValueError("bloch_spectral: alloy layers need the CPA form of bsf.f (api.bsf)")
    one = dataclasses.replace(ep, lg=ep.lg[:1], rg=ep.rg[:1])
    F, _ = S.layer_dos_inputs(ep, which)
    zero = np.zeros_like(F)
    kpts = np.asarray(kpts, float).reshape(-1, 2)
    al = np.zeros((len(kpts), ep.nintfc, ep.lmax + 1))
    aL = np.zeros((len(kpts), ep.nintfc, ep.lkmax))
    ctx = Context.for_problem(one)
    try:
        for i, k in enumerate(kpts):
            r = ctx.cpacoord(one.with_k(k[None, :], np.ones(1)))
            tm = r["tminv"]
            phys = np.array([N.phystau(r["tauc"][li], tm[li], ep.alpha[li], ep.lmax, ep.irel)
                             for li in range(ep.nintfc)])
            zm, zl = N.layer_dos(phys, F, zero, ep.lmax, ep.irel, para)
            al[i], aL[i] = zl.imag, zm.imag
    finally:
        ctx.close()
    return al, aL
