"""Energies staged up front in one context (skkr_gpu_stage_slot / run_slot)
give bit-identical results to the same energies in fresh contexts, on the
split-precision path with the FP64 redo of dominant k points: nothing of an
earlier energy (work buffers, split staging, freed compact buffers) leaks into
a later one.  The relativistic lmax=3 energies read the full (kappa,mu) pack
tables, whose last kappa has a spinor component outside the lm basis."""
import numpy as np
import pytest

from skkr_budapest_gb300 import api
from skkr_budapest_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run(ctx, slot):
    st = ctx.run_slot(slot, check=False)
    out = ctx.fetch_slot(slot) if st.code == 0 else None
    return st, out


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_slots_equal_fresh_contexts(precision):
    # unsplit wells under the 2 Ry / 0.7 d_NN barrier: these energies carry
    # isolated peaks of the k integrand, so the FP64 redo path runs
    spec = W.rel_bcc(so_split=0.0, vscreen=2.0, rscreen=0.7)
    order = [0, 12, 16, 4]
    eps = {ie: W.energy_problem(spec, ie) for ie in order}
    ctx = api.Context.for_problem(eps[order[0]], precision)
    try:
        ctx.set_mixed_policy(dominant_frac=1e-2)
        for i, ie in enumerate(order):
            ctx.stage_slot(i, eps[ie])
        seq = [_run(ctx, i) for i in range(len(order))]
    finally:
        ctx.close()
    redone = 0
    for i, ie in enumerate(order):
        st, out = seq[i]
        assert st.code == 0, (ie, st.code, st.ik)
        redone += st.k_fp64
        fresh = api.Context.for_problem(eps[ie], precision)
        try:
            fresh.set_mixed_policy(dominant_frac=1e-2)
            fresh.stage_slot(0, eps[ie])
            st2, out2 = _run(fresh, 0)
        finally:
            fresh.close()
        assert st2.code == 0
        assert st2.k_fp64 == st.k_fp64 and st2.inv_fallbacks == st.inv_fallbacks
        for key in ("tauc", "taua", "taub", "tminv"):
            assert np.array_equal(out[key], out2[key]), (ie, key)
    if precision == "mixed":
        assert redone > 0  # the redo path ran
