"""CPU reference of the Bloch spectral function of one interface layer (test
infrastructure: the checker of skkr_gpu_bsf, never the product path).

Restates skkr_dbogo_bsf/rsp-scf/bsf.f:140-420 for one layer and one k point:

* CPA layer (1 - c > tiny, bsf.f:140-158): species weights (c, 1 - c), the
  component taus tau_A, tau_B; D_a = tau_a tau_c^-1 and D~_a = tau_c^-1 tau_a
  (bsf.f:203-224); tau_diff = tau_c(k) - tau_c (bsf.f:238-240).
  Otherwise weights (1, 0) and tau_diff = tau_c(k) (bsf.f:155-157, 242).
* A0 (CPA layers only, bsf.f:251-276): sum_a c_a gf(a, a, tau_a).
* A1 (bsf.f:280-319): sum_ab c_a c_b gf(a, b, D_a tau_diff D~_b), with
  tau_diff itself in place of the triple product on a layer without CPA.
* gf (rsp-scf/gf.f:1-103 with reg = .true., gf.f:55-56: no irregular term) for solutions
  diagonal in the basis: ggrmat(j, i) = R_ab(j, i) X(j, i), R_ab the radial
  overlap of the right solution of species a at j with the left solution of
  species b at i (F on the diagonal of the electron and hole blocks, Feh on
  the electron-hole block; the other elements are never read below).
* Moments at lambda = 0 (rsp-scf/moment.f with the identity coefficient, as
  the layer DOS): zmat = -1/pi ggrmat; bsfe = sum over the electron
  diagonal of Im zmat, bsfh over the hole diagonal; for the four pairing
  operators P of rsp-scf/pairing.f (singlet, T0, T-up, T-down; gf.f:146-164
  trafogeh) Im tr(-1/pi P ggrmat_eh), in the order of bsf.f:366-418
  (bsfeh, bsfhe, bsfteh, bsfthe).

Plain numpy, FP64."""
from __future__ import annotations

import numpy as np

PAIRS = ("singlet", "t0", "tup", "tdown")


def gf_diag(F, Feh, a, b, X, nde):
    """ggrmat of gf.f for diagonal radial solutions: the electron and hole
    diagonals and the electron-hole block (None without BdG)."""
    nd = X.shape[0]
    diag = F[a, b, :nd] * np.diag(X)
    eh = None if Feh is None else Feh[a, b] * X[:nde, nde:]
    return diag, eh


def bsf_layer(tau_k, tau_c, tau_a, tau_b, conc, F, Feh=None, pair=None, tiny=1.0e-6, para=False, irel=1):
    """The six numbers of bsf.f for one layer at one k point:
    [bsfe, bsfh, bsfeh, bsfhe, bsfteh, bsfthe] (without BdG only bsfe).
    tau_* are physical (nd, nd) matrices; F (2, 2, nd), Feh (2, 2, nde, nde)
    the radial overlaps; pair the four (nde, nde) pairing operators."""
    nd = tau_k.shape[0]
    bdg = Feh is not None
    nde = nd // 2 if bdg else nd
    cpa = (1.0 - conc) > tiny
    diag = np.zeros(nd, complex)
    eh = np.zeros((nde, nde), complex) if bdg else None

    def add(w, a, b, X):
        d, e = gf_diag(F, Feh, a, b, X, nde)
        diag[:] += w * d
        if bdg:
            eh[:] += w * e

    if cpa:
        cab = (conc, 1.0 - conc)
        taui = (tau_a, tau_b)
        tinv = np.linalg.inv(tau_c)
        dmat = [t @ tinv for t in taui]
        dmatp = [tinv @ t for t in taui]
        tau_diff = tau_k - tau_c
        for a in range(2):
            add(cab[a], a, a, taui[a])                              # A0
            for b in range(2):
                add(cab[a] * cab[b], a, b, dmat[a] @ tau_diff @ dmatp[b])  # A1
    else:
        add(1.0, 0, 0, tau_k)
    fac = -1.0 / np.pi
    if para and irel == 0:
        fac *= 2.0
    out = np.zeros(6)
    out[0] = (fac * diag[:nde]).imag.sum()
    if bdg:
        out[1] = (fac * diag[nde:]).imag.sum()
        for x, name in enumerate(PAIRS):
            out[2 + x] = np.trace(fac * (pair[name] @ eh)).imag
    return out
