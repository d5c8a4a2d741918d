"""The reference's k-space form of the screened structure constants for a
workload energy: the inputs of skkr_gpu_stage_kambe.

main/gstore.f evaluates G_scr(k) per k point from the Kambe lattice sums of
every layer pair of a slab (kamstr.f) and screens the slab in k space
(scrstr.f, scrinv.f).  For a stacking of equivalent layers the slab is nl
consecutive layers of the stacking, every layer screened with the same
alpha, and the blocks the principal-layer packing reads are those of the
slab's central layer with its neighbours at the offsets of the table map.
"""
from __future__ import annotations

import math

import numpy as np


def square_lattice_vectors(a2d: float, gmax: float, rmax: float):
    """Reciprocal vectors with |g| <= gmax and direct vectors with |R| <= rmax
    of the square lattice of constant a2d (supersets: the sums skip terms
    beyond their own cut-offs)."""
    b = 2.0 * math.pi / a2d

    def pts(step, cut):
        n = int(cut / step) + 2
        i, j = np.meshgrid(np.arange(-n, n + 1), np.arange(-n, n + 1), indexing="ij")
        p = np.c_[i.ravel(), j.ravel()] * step
        return np.ascontiguousarray(p[np.hypot(p[:, 0], p[:, 1]) <= cut], np.float64)

    return pts(b, gmax), pts(a2d, rmax)


def kambe_form(ep, spec, nl: int = 8, centre: int | None = None, gcut: float = 12.0, rcut: float = 40.0,
               gmax: float = 14.0, rmax: float = 55.0, factor: float = 1.0) -> dict:
    """The arguments of skkr_gpu_stage_kambe for energy problem ep of system
    spec: the sums at the structure energy psq, a slab of nl layers of the
    stacking (kept block rows from layer `centre`, default nl // 2) screened
    with the interface alpha, the square lattice's vectors and cell area."""
    st = spec.stacking
    pos = np.ascontiguousarray([st.site(n, 0, 0) for n in range(nl)], np.float64)
    alpha = np.ascontiguousarray(np.array([ep.alpha[0][:ep.lmax + 1]] * nl, np.complex128))
    gvec, rvec = square_lattice_vectors(st.a2d, gmax, rmax)
    return dict(e=complex(ep.psq), nl=nl, pos=pos, alpha=alpha, centre=nl // 2 if centre is None else centre,
                gvec=gvec, rvec=rvec, area=st.a2d * st.a2d, factor=factor, gcut=gcut, rcut=rcut)
