"""Seeded workloads of the 2D-BZ tau path (one object per contour energy).

Each workload restates one benchmark configuration of the path with
synthetic inputs (see synth.py): a Bravais (001) stacking of identical square
layers, a semicircle contour, C4v IBZ k meshes with per-energy sizes, seeded
square-well t-matrices and real-space screened structure constants.

  plain_fcc   fcc(001) a=6.8, non-relativistic lmax=2 (9/site), PL2, 6-layer
              interface, 16 energies -0.5..0.7 Ry, 253 k per energy.
  rel_bcc     bcc(001) a=6.0, relativistic lmax=3 (32/site), PL4, 12-layer
              interface, 24 energies, 210..12090 k per energy (uneven),
              j = l +- 1/2 split wells, screening of the reference's bcc sample.
  rel_bcc_cpa rel_bcc with 4 alloy layers A_c B_(1-c).
  nonrel_pl2 / rel_pl3_l2   the two extra systems of the batched run.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import synth as S


@dataclass
class EnergyProblem:
    name: str
    ie: int
    ce: complex
    psq: complex
    fac: complex
    irel: int
    lmax: int
    lkmax: int
    nprc: int
    ninprc: np.ndarray          # int32 (nprc+2,)
    bulkgeo: int
    nintfc: int
    blkmap: np.ndarray          # int32 (nslot, mi, 2*jmax+1)
    rt: S.RTable
    xk: np.ndarray              # (nk, 2)
    wk: np.ndarray              # (nk,)
    lg: np.ndarray              # (ngeff, lk, lk)
    rg: np.ndarray
    tminvl: np.ndarray          # (ninprc[0], lk, lk)
    tminvr: np.ndarray          # (ninprc[-1], lk, lk)
    tminv: np.ndarray           # (nintfc, lk, lk)  initial coherent (ATA for alloys)
    tminva: np.ndarray
    tminvb: np.ndarray
    conc: np.ndarray            # (nintfc,)
    alpha: np.ndarray           # (nintfc, lmax+1) screening per interface layer (BdG: alpha_e, alpha_h)
    itermaxl: int = 50
    itermaxr: int = 50
    errmax: float = 1.0e-8
    itcpam: int = 50
    cpatol: float = 1.0e-10
    meta: dict = field(default_factory=dict)
    rt_h: S.RTable | None = None    # BdG: hole structure-constant table (same R vectors as rt)
    fach: complex = 0.0             # BdG: relmtrx factor of the hole block

    @property
    def nk(self) -> int:
        return len(self.xk)

    @property
    def n_pl(self) -> int:
        return int(max(self.ninprc)) * self.lkmax

    def with_k(self, xk, wk) -> "EnergyProblem":
        import copy
        c = copy.copy(self)
        c.xk = np.ascontiguousarray(xk, float)
        c.wk = np.ascontiguousarray(wk, float)
        return c


@dataclass
class SystemSpec:
    name: str
    stacking: S.Stacking
    irel: int
    lmax: int
    pl: int                   # layers per principal layer
    nprc: int
    energies: np.ndarray
    nsets: list               # per energy IBZ subdivision
    seed: int
    depth_range: tuple = (-1.0, -0.5)
    radius: float = 2.5
    so_split: float = 0.03
    vscreen: float = 2.0
    rscreen: float = 0.7      # radius of the screening spheres in units of the NN distance
    alloy_layers: tuple = ()
    conc_range: tuple = (0.1, 0.9)
    alloy_depth_range: tuple = (-1.2, -0.4)
    cpatol: float = 1.0e-10
    # neighbour shells of the cluster the screening inversion runs on (the
    # table keeps 3 shells): on the bare 3-shell cluster the boundary distorts
    # the kept couplings enough that the lead decimation of the bcc stacking
    # exceeds the 1e10 limit of surfgf.f at the contour points nearest the axis
    screen_shells: int = 5
    # BdG (irel=2): energies relative to e_fermi, pairing delta on sc_layers
    # (interface layer indices) and on the leads flagged in sc_leads (L, R)
    e_fermi: float = 0.0
    delta: float = 0.0
    sc_layers: tuple = ()
    sc_leads: tuple = (False, False)


def _contour(ne, eb, et, eps):
    z, _ = S.zmesh_semicircle(ne, eb, et, eps)
    return z


def plain_fcc(nset: int = 22) -> SystemSpec:
    return SystemSpec("plain_fcc", S.fcc001(6.8), 0, 2, 2, 3, _contour(16, -0.5, 0.7, 150.0),
                      [nset] * 16, seed=0)


# per-energy IBZ subdivisions of the relativistic interface: 210 k far from the
# real axis up to 12090 k at the contour point nearest E_F (Im E = 5e-4 Ry),
# grouped like the reference's KSETTAB/INTAB table
REL_NSETS = [20] * 12 + [32] * 4 + [48] * 3 + [70] * 2 + [100, 125, 155]


# Screening of the bcc(001) workloads: the reference's own bcc layer sample
# (sample/02-layer-scf: ISCREEN 1, VSCREEN 3.0 Ry, screening spheres of the
# Wigner-Seitz radius, sws = 3.0709 a.u. of its Nb) -- 3 Ry in spheres of the
# bcc Wigner-Seitz radius, r_WS / d_NN = (3 / (8 pi))^(1/3) / (sqrt(3) / 2).
# With it the three-shell screened table is localised and the lead
# decimation of the j = l +- 1/2 split wells stays below surfgf.f's 1e10
# limit on every contour energy and mesh; the 2 Ry / 0.7 d_NN barrier of the
# fcc configuration does neither for the split bcc lead.
WS_BCC = (3.0 / (8.0 * math.pi)) ** (1.0 / 3.0) / (math.sqrt(3.0) / 2.0)


def rel_bcc(nsets=None, so_split: float = 0.03, vscreen: float = 3.0, rscreen: float = WS_BCC) -> SystemSpec:
    """The relativistic PL4 lmax=3 interface: j = l +- 1/2 split wells
    (0.03 Ry <l.s>), the reference sample's bcc screening."""
    z = _contour(24, -0.5, 0.7, 10.0)
    return SystemSpec("rel_bcc", S.bcc001(6.0), 1, 3, 4, 3, z,
                      list(REL_NSETS if nsets is None else nsets), seed=1, so_split=so_split, vscreen=vscreen,
                      rscreen=rscreen)


def rel_bcc_cpa(nsets=None, so_split: float = 0.03) -> SystemSpec:
    s = rel_bcc(nsets, so_split)
    s.name = "rel_bcc_cpa"
    s.seed = 2
    s.alloy_layers = (4, 5, 6, 7)
    return s


def nonrel_pl2() -> SystemSpec:
    z = _contour(16, -0.5, 0.7, 10.0)
    return SystemSpec("nonrel_pl2", S.fcc001(6.8), 0, 2, 2, 3, z,
                      [14] * 8 + [20] * 4 + [40] * 2 + [80, 126], seed=3)


def rel_pl3_l2(so_split: float = 0.03) -> SystemSpec:
    z = _contour(20, -0.5, 0.7, 10.0)
    return SystemSpec("rel_pl3_l2", S.bcc001(6.0), 1, 2, 3, 3, z,
                      [14] * 10 + [20] * 4 + [40] * 3 + [60, 90, 126], seed=4, so_split=so_split, vscreen=3.0,
                      rscreen=WS_BCC)


def bdg_bcc(nsets=None, lmax: int = 3, pl: int = 4, ne: int = 64, im_e: float = 1.0e-4) -> SystemSpec:
    """BdG interface (skkr_dbogo_bsf layout: electron (kappa,mu) block then hole
    block, 4 (lmax+1)^2 per site): bcc(001) a=6.0, PL4 (n_PL = 256 at lmax=3),
    3 interface PLs; superconducting left lead and first half of the interface
    (delta = 1e-3 Ry), normal right lead and second half.  ne energies at
    Im E = im_e spread over +-5 delta around E_F = 0.7 Ry."""
    delta = 1.0e-3
    z = np.linspace(-5 * delta, 5 * delta, ne) + 1j * im_e
    nintfc = pl * 3
    return SystemSpec("bdg_bcc", S.bcc001(6.0), 2, lmax, pl, 3, z,
                      list([6] * ne if nsets is None else nsets), seed=5, e_fermi=0.7, delta=delta,
                      sc_layers=tuple(range(nintfc // 2)), sc_leads=(True, False), so_split=0.0)


def system_layers(spec: SystemSpec):
    ninprc = np.array([spec.pl] * (spec.nprc + 2), np.int32)
    return ninprc, spec.pl * spec.nprc


def screened_table(spec: SystemSpec, ie: int):
    """G_scr(R) of contour point ie (non-BdG): the screened real-space table
    the GPU path Fourier-transforms per k, built on the host."""
    ce = complex(spec.energies[ie])
    psq = ce + ce * ce / (S.C_LIGHT * S.C_LIGHT) if spec.irel else ce
    _, _, dnn = S.cluster(spec.stacking, 1)
    alpha = S.alpha_sqwell(ce, spec.vscreen, spec.rscreen * dnn, spec.lmax)
    return S.build_rtable(spec.stacking, psq, alpha, spec.lmax, nshell_screen=spec.screen_shells)


def _table_seconds(job):
    import time
    spec, ie = job
    t = time.perf_counter()
    screened_table(spec, ie)
    return time.perf_counter() - t


def table_build_seconds(spec: SystemSpec, energies, workers: int) -> float:
    """Wall time to build the screened tables of `energies` on `workers` host
    processes (spawned: the caller may already hold a CUDA context)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os
    import time
    if workers <= 1:
        t = time.perf_counter()
        for ie in energies:
            screened_table(spec, ie)
        return time.perf_counter() - t
    keep = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in keep:
        os.environ[k] = "1"   # one BLAS thread per worker process
    try:
        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            list(ex.map(_table_seconds, [(spec, energies[0])] * workers))   # start-up outside the timing
            t = time.perf_counter()
            list(ex.map(_table_seconds, [(spec, ie) for ie in energies]))
            return time.perf_counter() - t
    finally:
        for k, v in keep.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def energy_problem(spec: SystemSpec, ie: int, nset: int | None = None, kmesh: str = "ibz") -> EnergyProblem:
    """Build the inputs of contour point ie of a system (seeded, deterministic)."""
    if spec.irel == 2:
        return _bdg_problem(spec, ie, nset, kmesh)
    ce = complex(spec.energies[ie])
    lmax = spec.lmax
    irel = spec.irel
    if irel:
        psq = ce + ce * ce / (S.C_LIGHT * S.C_LIGHT)
        lk = 2 * (lmax + 1) ** 2
    else:
        psq = ce
        lk = (lmax + 1) ** 2
    fac = psq / ce
    st = spec.stacking
    _, _, dnn = S.cluster(st, 1)
    alpha = S.alpha_sqwell(ce, spec.vscreen, spec.rscreen * dnn, lmax)
    rt = screened_table(spec, ie)
    ninprc, nintfc = system_layers(spec)
    blkmap = S.blkmap_translation_invariant(rt, spec.nprc + 2, int(max(ninprc)))

    rng = np.random.default_rng(spec.seed)
    d_bulk = rng.uniform(*spec.depth_range)
    d_int = rng.uniform(*spec.depth_range, size=nintfc)
    conc = np.ones(nintfc)
    d_a = d_int.copy()
    d_b = d_int.copy()
    for li in spec.alloy_layers:
        conc[li] = rng.uniform(*spec.conc_range)
        d_a[li] = rng.uniform(*spec.alloy_depth_range)
        d_b[li] = rng.uniform(*spec.alloy_depth_range)

    def tinv(depth):
        if irel:
            return S.screened_tinv_rel(ce, psq, depth, spec.radius, spec.so_split, alpha, lmax)
        return S.screened_tinv_nonrel(ce, depth, spec.radius, alpha, lmax)

    tb = tinv(d_bulk)
    tminvl = np.array([tb] * ninprc[0])
    tminvr = np.array([tb] * ninprc[-1])
    ta = np.array([tinv(d) for d in d_a])
    tbb = np.array([tinv(d) for d in d_b])
    tm = ta.copy()
    for li in spec.alloy_layers:
        tm[li] = ata(conc[li], ta[li], tbb[li])

    ns = spec.nsets[ie] if nset is None else nset
    if kmesh == "ibz":
        xk, wk = S.kmesh_square_c4v(ns, st.a2d)
        lg, rg = S.point_group_mats(lmax, irel)
    else:
        xk, wk = S.kmesh_square_full(ns, st.a2d)
        lg, rg = S.point_group_mats(lmax, irel)
        lg, rg = lg[:1], rg[:1]
    return EnergyProblem(spec.name, ie, ce, psq, fac, irel, lmax, lk, spec.nprc, ninprc, 1, nintfc,
                         blkmap, rt, xk, wk, lg, rg, tminvl, tminvr, tm, ta, tbb, conc,
                         np.array([alpha] * nintfc), cpatol=spec.cpatol,
                         meta=dict(nset=ns, depth_bulk=d_bulk, depth_a=d_a, depth_b=d_b,
                                   radius=spec.radius, so_split=spec.so_split))


def _bdg_problem(spec: SystemSpec, ie: int, nset, kmesh) -> EnergyProblem:
    """Energy point of a BdG system, with the electron/hole energies and
    factors of skkr_dbogo_bsf rsp-scf/cpacoord_ksave.f:160-169:
    celoc = E_F + E, fac = psq/celoc; celoch = E_F - conj(E),
    fach = conj(psqh)/conj(celoch)."""
    c = S.C_LIGHT
    ce = complex(spec.energies[ie])
    ef = spec.e_fermi
    celoc = ef + ce
    psq = celoc + celoc * celoc / (c * c)
    fac = psq / celoc
    celoch = ef - ce.conjugate()
    psqh = celoch + celoch * celoch / (c * c)
    fach = psqh.conjugate() / celoch.conjugate()
    lmax = spec.lmax
    lk = 4 * (lmax + 1) ** 2
    st = spec.stacking
    _, _, dnn = S.cluster(st, 1)
    rs = spec.rscreen * dnn
    alpha_e = S.alpha_sqwell(psq, spec.vscreen, rs, lmax)
    alpha_h = S.alpha_sqwell_hole(ef - ce, spec.vscreen, rs, lmax)
    rt = S.build_rtable(st, psq, alpha_e, lmax, nshell_screen=spec.screen_shells)
    rt_h = S.build_rtable(st, psqh, alpha_h, lmax, hole=True, nshell_screen=spec.screen_shells)
    ninprc, nintfc = system_layers(spec)
    blkmap = S.blkmap_translation_invariant(rt, spec.nprc + 2, int(max(ninprc)))
    rng = np.random.default_rng(spec.seed)
    d_bulk_l, d_bulk_r = rng.uniform(*spec.depth_range, size=2)
    d_int = rng.uniform(*spec.depth_range, size=nintfc)

    def tinv(depth, sc):
        return S.bdg_tinv(celoc, psq, celoch, psqh, depth, spec.radius, spec.so_split, alpha_e, alpha_h,
                          lmax, spec.delta if sc else 0.0)

    tl = tinv(d_bulk_l, spec.sc_leads[0])
    tr = tinv(d_bulk_r, spec.sc_leads[1])
    tm = np.array([tinv(d, li in spec.sc_layers) for li, d in enumerate(d_int)])
    ns = spec.nsets[ie] if nset is None else nset
    # electron block transforms with D, the hole block (structure constants
    # after lmtolmconj) with D*: blockdiag(D, D*) (the reference's sphbas.f
    # uses blockdiag(D, D), which only holds while the blocks decouple)
    lg1, rg1 = S.point_group_mats(lmax, 1)
    z = np.zeros_like(lg1)
    lg = np.block([[lg1, z], [z, lg1.conj()]])
    rg = np.block([[rg1, z], [z, rg1.conj()]])
    if kmesh == "ibz":
        xk, wk = S.kmesh_square_c4v(ns, st.a2d)
    else:
        xk, wk = S.kmesh_square_full(ns, st.a2d)
        lg, rg = lg[:1], rg[:1]
    return EnergyProblem(spec.name, ie, ce, psq, fac, 2, lmax, lk, spec.nprc, ninprc, 1, nintfc,
                         blkmap, rt, xk, wk, lg, rg, np.array([tl] * ninprc[0]), np.array([tr] * ninprc[-1]),
                         tm, tm.copy(), tm.copy(), np.ones(nintfc),
                         np.array([np.concatenate([alpha_e, alpha_h])] * nintfc), cpatol=spec.cpatol,
                         meta=dict(nset=ns, celoc=celoc, celoch=celoch, psqh=psqh, depth_int=d_int,
                                   radius=spec.radius, so_split=spec.so_split),
                         rt_h=rt_h, fach=fach)


def ata(conc: float, ma: np.ndarray, mb: np.ndarray) -> np.ndarray:
    """rsp-scf/fullcpa.f:2-23 tata: m_c = m_B (c m_B + (1-c) m_A)^-1 m_A."""
    mc = conc * mb + (1.0 - conc) * ma
    return mb @ np.linalg.inv(mc) @ ma
