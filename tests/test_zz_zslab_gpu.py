"""The reference's screened G_scr(k) on the device (skkr_gpu_kambe_screened:
layer-pair blocks of a slab from the Kambe sums, 1 - alpha G inverted per k
by the batched Gauss-Jordan kernel, times G by the batched GEMM, the central
layer offsets extracted) against the oracle's gstore + scrstr restatement
(oracle/kambe.py screened_slab), with a barrier that localises the screened
constants."""
import numpy as np
import pytest

import kambe as K
from skkr_budapest_gb300 import native
from skkr_budapest_gb300 import synth as S
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_screened_slab_on_the_device_matches_the_oracle():
    spec = W.plain_fcc(nset=4)
    st = spec.stacking
    lat = K.Lattice2D([st.a2d, 0.0], [0.0, st.a2d])
    _, _, dnn = S.cluster(st, 1)
    ce = complex(spec.energies[8])
    al = S.alpha_sqwell(ce, 4.0, 0.5 * dnn, spec.lmax)
    nl, centre, jmax = 8, 4, 2
    pos = np.array([st.site(n, 0, 0) for n in range(nl)])
    kpts = [(0.31, 0.12), (0.0, 0.0), (0.5, 0.2)]
    dev = native.kambe_screened(ce, kpts, pos, [al] * nl, spec.lmax, lat.gvecs(14.0), lat.rvecs(55.0), lat.area,
                                centre, jmax)
    for i, k in enumerate(kpts):
        gs = K.screened_slab(ce, k[0], k[1], spec.lmax, pos, [al] * nl, lat)
        ref = np.array([gs[centre, centre + j] for j in range(-jmax, jmax + 1)])
        assert np.abs(dev[i] - ref).max() < 1e-10 * np.abs(ref).max(), k
