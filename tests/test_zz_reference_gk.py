"""The reference's k-space structure constants on the device, one thread per
(k point, separation) item: the Kambe lattice sums of main/kamstr.f
(skkr_gpu_kambe_dlm) against the oracle's restatement on the same lattice
vectors, and the layer-pair blocks they contract to (skkr_gpu_kambe_alm)
against the oracle's kamstr, at energies down to Im E = 1e-4 Ry and for the
zero, in-plane and out-of-plane separations of the layer pairs."""
import numpy as np
import pytest

import kambe as K
from skkr_budapest_gb300 import native

pytestmark = pytest.mark.gpu

A2D = 4.808326112068523
LAT = K.Lattice2D([A2D, 0.0], [0.0, A2D])
SEPS = [(0.0, 0.0, 0.0), (1.2, 0.7, 3.4), (0.5 * A2D, 0.5 * A2D, 0.0), (0.4, -1.1, -6.8)]
KS = [(0.21, 0.07), (0.0, 0.0), (0.6, 0.31)]


@pytest.mark.parametrize("e", [0.3 + 0.01j, -0.45 + 0.06j, 0.7 + 1e-4j])
@pytest.mark.parametrize("lmax2", [4, 6])
def test_device_kambe_sums_match_the_oracle(e, lmax2):
    items = [(k, s) for k in KS for s in SEPS]
    g = LAT.gvecs(14.0)
    r = LAT.rvecs(55.0)
    d = native.kambe_dlm(e, [k for k, _ in items], [s for _, s in items], lmax2, g, r, LAT.area)
    for i, (k, s) in enumerate(items):
        ref = K.kambe_dlm(e, *k, s, lmax2, LAT, gcut=12.0, rcut=40.0)
        # in plane the recursion of delkam amplifies rounding by ~1e6 (kamstr's
        # s_z = 1.1e-4 shift): a host build with fused multiply-adds already
        # parts from the oracle by 7e-10 there, against the shift's own 8e-5
        in_plane = s[2] == 0.0 and any(s[:2])
        assert np.abs(d[i] - ref).max() < (1e-8 if in_plane else 1e-12) * np.abs(ref).max(), (k, s)


@pytest.mark.parametrize("e", [0.3 + 0.01j, 0.7 + 1e-4j])
@pytest.mark.parametrize("lmax", [2, 3])
def test_device_layer_pair_blocks_match_kamstr(e, lmax):
    items = [(k, s) for k in KS[:2] for s in SEPS]
    g = LAT.gvecs(14.0)
    r = LAT.rvecs(55.0)
    a = native.kambe_alm(e, [k for k, _ in items], [s for _, s in items], lmax, g, r, LAT.area)
    for i, (k, s) in enumerate(items):
        ref = K.kamstr(e, *k, lmax, s, LAT, gcut=12.0, rcut=40.0)
        in_plane = s[2] == 0.0 and any(s[:2])
        assert np.abs(a[i] - ref).max() < (1e-8 if in_plane else 1e-12) * np.abs(ref).max(), (k, s)
