"""Screened real-space structure constants of the input generator (CPU).

G_scr = G0 (1 - alpha G0)^-1 on a cluster, alpha the square-well t-matrix of
main/alphamat.f.  With a barrier that screens (4 Ry in touching spheres,
radius d_NN / 2), the constants of the first three shells decay and stop
depending on the size of the cluster the inversion runs on; the same barrier
with the sign of alpha flipped does not localise them.  This pins the sign
convention of alpha against the free-space G0."""
import numpy as np

from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W


def _tables(alpha_sign, ie):
    spec = W.plain_fcc(nset=4)
    st = spec.stacking
    _, _, dnn = S.cluster(st, 1)
    ce = complex(spec.energies[ie])
    alpha = alpha_sign * S.alpha_sqwell(ce, 4.0, 0.5 * dnn, spec.lmax)
    n3 = len(S.cluster(st, 3)[0])
    out = {}
    for ns in (5, 9):
        big, _, _ = S.cluster(st, ns)
        out[ns] = S.screened_realspace(ce, big, alpha, spec.lmax)
    return out, n3


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_screening_localises_the_constants():
    for ie in (0, 8, 15):
        t, n3 = _tables(+1, ie)
        assert _rel(t[5][:n3], t[9][:n3]) < 1e-3
        # decay over the 9-shell cluster: the 5th shell far below the 1st
        big, _, _ = S.cluster(W.plain_fcc(nset=4).stacking, 9)
        d = np.round(np.linalg.norm(big, axis=1), 5)
        shells = np.unique(d)
        first = max(np.linalg.norm(t[9][i]) for i in np.where(d == shells[1])[0])
        fifth = max(np.linalg.norm(t[9][i]) for i in np.where(d == shells[5])[0])
        assert fifth < 1e-2 * first


def test_flipped_alpha_does_not_localise():
    t, n3 = _tables(-1, 8)
    assert _rel(t[5][:n3], t[9][:n3]) > 1e-1
