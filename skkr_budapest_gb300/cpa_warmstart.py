"""Learned warm start of the CPA loop (the C4 surrogate).

The CPA iteration of rsp-scf/fullcpa.f (cpacor/cpasol) starts from the
coherent inverse t-matrix m_c it is given: the ATA average (tata,
fullcpa.f:2-23) or an effective t-matrix read back from a previous run
(main/tcpaio.f:193-276).  Here a network trained on converged CPA solutions
of the method itself predicts m_c; the CPA iteration is unchanged (same
update, same error3 test, same tolerance), only its starting point moves, so
the converged result is the same up to the CPA tolerance.

The system family (C4): the relativistic bcc(001) PL4 lmax=3 interface of
the benchmarked workload with 4 alloy layers A_c B_(1-c); every other layer
and the leads are fixed, each alloy layer draws c ~ U[0.1, 0.9] and square-
well depths of A and B ~ U[-1.2, -0.4] Ry.  The coherent t-matrix of one
alloy layer depends on the whole alloy stack, so the inputs of one sample
(one alloy layer at one energy) are

    Re E, Im E, the layer's position (one-hot over the 4 alloy layers),
    then for the layer itself and the other alloy layers in stack order:
    c, Re/Im of the kappa-diagonal of m_A and of m_B

(E, c and the diagonals of t_A / t_B, the C4 inputs, for the whole stack).
The output is the correction of the converged m_c to the ATA start on the
elements the point group leaves free (the matrices with R_g m L_g = m for
all g; 256 of the 32 x 32 elements at lmax=3), divided by the layer's mean
|m_A - m_B| over kappa.  The warm start is m_ATA + the prediction projected
onto those invariant matrices.

The network is 3 tanh hidden layers of 256 with BF16 weights and FP32
accumulation, trained and evaluated by this library's own kernels
(skkr_gpu_mlp16_*: forward, backward, AdamW on FP32 masters).

    python -m skkr_budapest_gb300.cpa_warmstart gen   --out data.npz   (GPU)
    python -m skkr_budapest_gb300.cpa_warmstart train --data data.npz  (GPU)
    python -m skkr_budapest_gb300.cpa_warmstart report                 (GPU)
"""
from __future__ import annotations

import argparse
import copy
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import synth as S
from . import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "data", "cpa_surrogate_c4.npz")
HIDDEN = (256, 256, 256)


@dataclass
class Family:
    """The C4 alloy interface family: host system fixed, alloy stack drawn."""
    nset: int = 6                      # IBZ subdivision of the k mesh of every energy
    host_seed: int = 2                 # leads and non-alloy layers (rel_bcc_cpa's seed)
    so_split: float = 0.03             # j = l +- 1/2 split of the well depths, as the C2 interface
    lmax: int = 3
    alloy_layers: tuple = (4, 5, 6, 7)
    conc_range: tuple = (0.1, 0.9)
    depth_range: tuple = (-1.2, -0.4)
    # the contour energies with Im E >= 0.013 Ry: nearer the axis a mesh this
    # coarse leaves the CPA iteration itself stalling above 1e-10 (from any start)
    energies: tuple = tuple(range(21))
    _base: dict = field(default_factory=dict, repr=False)

    def spec(self):
        s = W.rel_bcc_cpa(so_split=self.so_split)
        s.seed = self.host_seed
        s.lmax = self.lmax
        s.nsets = [self.nset] * len(s.energies)
        return s

    def base(self, ie: int):
        """The EnergyProblem of contour energy ie with the host's own alloy
        draw (its table and leads are what every configuration shares)."""
        if ie not in self._base:
            self._base[ie] = W.energy_problem(self.spec(), ie)
        return self._base[ie]

    def draw(self, rng):
        na = len(self.alloy_layers)
        return (rng.uniform(*self.conc_range, na), rng.uniform(*self.depth_range, na),
                rng.uniform(*self.depth_range, na))

    def problem(self, ie: int, cfg):
        """Energy ie with the alloy stack cfg = (c, depth_A, depth_B): species
        t^-1 of the drawn wells, ATA start (tata) on the alloy layers."""
        b = self.base(ie)
        ep = copy.copy(b)
        conc, da, db = cfg
        ep.conc = b.conc.copy()
        ep.tminva, ep.tminvb, ep.tminv = b.tminva.copy(), b.tminvb.copy(), b.tminv.copy()
        alpha = b.alpha[0]
        for j, li in enumerate(self.alloy_layers):
            ta = S.screened_tinv_rel(b.ce, b.psq, da[j], b.meta["radius"], self.so_split, alpha, self.lmax)
            tb = S.screened_tinv_rel(b.ce, b.psq, db[j], b.meta["radius"], self.so_split, alpha, self.lmax)
            ep.conc[li] = conc[j]
            ep.tminva[li], ep.tminvb[li] = ta, tb
            ep.tminv[li] = W.ata(conc[j], ta, tb)
        ep.meta = dict(b.meta, cfg=cfg)
        return ep


class _KGroups:
    """The (kappa,mu) basis grouped by kappa (clebsch.f order): the index
    arrays, and the same as one permutation with group starts and sizes for
    the per-group means."""

    def __init__(self, lmax: int):
        _, kv = S.kmy_l_kappa(lmax)
        kappas = []
        for k in kv.tolist():
            if k not in kappas:
                kappas.append(k)
        self.groups = [np.nonzero(kv == k)[0] for k in kappas]
        self.order = np.concatenate(self.groups)
        self.sizes = np.array([len(g) for g in self.groups], float)
        self.starts = np.concatenate([[0], np.cumsum([len(g) for g in self.groups])[:-1]])


_KG: dict = {}


def kappa_groups(lmax: int) -> _KGroups:
    if lmax not in _KG:
        _KG[lmax] = _KGroups(lmax)
    return _KG[lmax]


def _kdiag(m, groups: _KGroups):
    """Mean of the diagonal of m over each kappa group."""
    d = np.diag(m)[groups.order]
    return np.add.reduceat(d, groups.starts) / groups.sizes


def invariant_projector(ep):
    """P(m) = (1/ng) sum_g R_g m L_g: the point-group average under which the
    k-summed tau and hence the converged m_c are invariant."""
    lg, rg = np.asarray(ep.lg), np.asarray(ep.rg)
    return lambda m: (rg @ m @ lg).mean(axis=0)


def projector_matrix(ep, mask):
    """The point-group average P restricted to the free elements: the
    (n*n, nfree) matrix whose column f is P of the unit matrix at the f-th
    True entry of mask (row-major), so that P(d) = (Pm @ d[mask]) for every d
    that vanishes off the mask."""
    lg, rg = np.asarray(ep.lg), np.asarray(ep.rg)
    j, k = np.nonzero(mask)
    pm = np.einsum("gif,gfm->imf", rg[:, :, j], lg[:, k, :]) / len(lg)
    return pm.reshape(-1, len(j))


def free_elements(ep):
    """Mask of the matrix elements that invariant matrices can carry."""
    P = invariant_projector(ep)
    n = ep.lkmax
    rng = np.random.default_rng(0)
    acc = np.zeros((n, n))
    for _ in range(3):
        acc += np.abs(P(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))))
    return acc > 1e-9 * acc.max()


def stack_features(ep, fam: Family):
    """One input row per alloy layer (see the module docstring)."""
    groups = kappa_groups(fam.lmax)
    al = list(fam.alloy_layers)
    per = {}
    for li in al:
        ma, mb = _kdiag(ep.tminva[li], groups), _kdiag(ep.tminvb[li], groups)
        per[li] = np.concatenate([[ep.conc[li]], ma.real, ma.imag, mb.real, mb.imag])
    rows = []
    for j, li in enumerate(al):
        onehot = np.zeros(len(al))
        onehot[j] = 1.0
        order = [li] + [x for x in al if x != li]
        rows.append(np.concatenate([[ep.ce.real, ep.ce.imag], onehot] + [per[x] for x in order]))
    return np.array(rows)


def _scale(ep, li, groups):
    return np.abs(_kdiag(ep.tminva[li], groups) - _kdiag(ep.tminvb[li], groups)).mean() + 1e-30


def _scales(ep, layers, groups):
    """_scale of each of the layers, all at once."""
    d = np.diagonal(ep.tminva[layers] - ep.tminvb[layers], axis1=1, axis2=2)[:, groups.order]
    return np.abs(np.add.reduceat(d, groups.starts, axis=1) / groups.sizes).mean(axis=1) + 1e-30


def stack_targets(ep, mc, fam: Family, mask):
    """(m_c - m_ATA) on the free elements, Re then Im, over the layer's scale."""
    groups = kappa_groups(fam.lmax)
    out = []
    for li in fam.alloy_layers:
        d = (mc[li] - ep.tminv[li])[mask] / _scale(ep, li, groups)
        out.append(np.concatenate([d.real, d.imag]))
    return np.array(out)


def bf16_round(a):
    """Nearest BF16 value (ties to even) of the FP32 value of each entry."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


class Model:
    """The trained surrogate: FP32 master layers, input and output
    normalisation, the free-element mask."""

    def __init__(self, path: str = DEFAULT_MODEL):
        z = np.load(path)
        self.layers = [(z["w%d" % i].astype(np.float32), z["b%d" % i].astype(np.float32))
                       for i in range(int(z["nlayers"]))]
        self.xmean, self.xstd = z["xmean"], z["xstd"]
        self.ymean, self.ystd = z["ymean"], z["ystd"]
        self.mask = z["mask"].astype(bool)
        self.nset = int(z["nset"])
        self.so_split = float(z["so_split"])
        self.info = {k: z[k] for k in z.files if k.startswith(("train_", "val_", "n_"))}

    def predict(self, x, device: str = "gpu"):
        """Normalised outputs -> targets.  device "gpu": the library's BF16
        forward kernel; "host": the same network in numpy (rounded weights,
        FP32 arithmetic), for machines without a GPU."""
        h = np.float32((np.atleast_2d(x) - self.xmean) / self.xstd)
        if device == "gpu":
            from . import native as N
            if getattr(self, "_net", None) is None or len(h) > self._net.maxrows:
                self._net = N.Mlp16Net(self.layers, max(64, len(h)))
            y = self._net(h)
        else:
            if getattr(self, "_w16", None) is None:
                self._w16 = [bf16_round(w) for w, _ in self.layers]
            y = h
            for i, (w, (_, b)) in enumerate(zip(self._w16, self.layers)):
                y = np.float32(y @ w + b)
                if i < len(self.layers) - 1:
                    y = np.tanh(y)
        return y * self.ystd + self.ymean

    def family(self):
        return Family(nset=self.nset, so_split=self.so_split)

    def projector(self, ep):
        """projector_matrix of ep on the model's mask, built once per set of
        group matrices: every energy of one lattice carries equal ones (as
        separate arrays), found by identity and else by value."""
        cache = self.__dict__.setdefault("_proj", [])
        for lg, rg, pm in cache:
            if lg is ep.lg and rg is ep.rg:
                return pm
        for lg, rg, pm in cache:
            if np.array_equal(lg, ep.lg) and np.array_equal(rg, ep.rg):
                cache.append((ep.lg, ep.rg, pm))
                del cache[:-32]
                return pm
        pm = projector_matrix(ep, self.mask)
        cache.append((ep.lg, ep.rg, pm))
        del cache[:-32]
        return pm


def warm_start(ep, model: Model, fam: Family | None = None, device: str = "gpu"):
    """Starting coherent t^-1: m_ATA + the projected prediction on the alloy
    layers of the family, the given start elsewhere."""
    fam = fam or model.family()
    groups = kappa_groups(fam.lmax)
    pred = model.predict(stack_features(ep, fam), device)
    al = list(fam.alloy_layers)
    pm = model.projector(ep)
    nm = int(model.mask.sum())
    d = (pred[:, :nm] + 1j * pred[:, nm:2 * nm]) * _scales(ep, al, groups)[:, None]
    tm = np.array(ep.tminv, copy=True)
    tm[al] += (d @ pm.T).reshape(len(al), *tm.shape[1:])
    return tm


def generate(out: str, nsolve: int, fam: Family, seed: int = 1000, precision: str = "mixed", nctx: int = 8,
             max_seconds: float = 1e9, graphs: bool = True, progress: int = 50):
    """Converged CPA solutions of nsolve drawn alloy stacks, energies cycled
    over the contour, nctx systems per call (skkr_gpu_cpacoord_many).  Saves
    x [rows, 122], y [rows, 2 nfree], solve id, energy, CPA iterations."""
    from . import api
    rng = np.random.default_rng(seed)
    mask = free_elements(fam.base(fam.energies[0]))
    ctxs = [api.Context.for_problem(fam.base(fam.energies[0]), precision) for _ in range(nctx)]
    for c in ctxs:
        c.set_graphs(graphs)
    xs, ys, meta = [], [], []
    t0 = time.time()
    s = 0
    try:
        while s < nsolve and time.time() - t0 < max_seconds:
            group = []
            for _ in range(min(nctx, nsolve - s)):
                ie = fam.energies[s % len(fam.energies)]
                group.append((s, ie, fam.problem(ie, fam.draw(rng))))
                s += 1
            res = api.cpacoord_many([g[2] for g in group], contexts=ctxs[:len(group)], check=False)
            for (sid, ie, ep), r in zip(group, res):
                if r["status"] != 0 or r["cpa_error"] > ep.cpatol:
                    continue
                xs.append(stack_features(ep, fam))
                ys.append(stack_targets(ep, r["tminv"], fam, mask))
                meta += [(sid, ie, li, r["cpa_iterations"]) for li in fam.alloy_layers]
            if s % (progress * nctx) < nctx:
                print("%d solves, %d rows, %.1f s" % (s, 4 * len(xs), time.time() - t0), flush=True)
    finally:
        for c in ctxs:
            c.close()
    np.savez(out, x=np.concatenate(xs).astype(np.float32), y=np.concatenate(ys).astype(np.float32),
             meta=np.array(meta, np.int32), mask=mask, nset=fam.nset, so_split=fam.so_split,
             seconds=time.time() - t0)
    return len(meta)


def train(data: str, out: str, schedule=((4000, 1e-3), (4000, 3e-4), (4000, 1e-4)), weight_decay: float = 0.0,
          seed: int = 0, val_frac: float = 0.1, eval_every: int = 25, norm: str = "global"):
    """Full-batch AdamW of the BF16-weight network on the device
    (skkr_gpu_mlp16_train) in phases of (epochs, learning rate), each phase
    restarting from the previous phase's best held-out parameters; the last
    val_frac of the solves is held out.  norm "global": one output scale (the
    loss is the mean squared error of the correction itself); "column": every
    output standardised.  Returns (train mse, held-out mse, held-out mse of the
    ATA start), in units of the targets."""
    from . import native as N
    z = np.load(data)
    x, y, meta = z["x"].astype(np.float64), z["y"].astype(np.float64), z["meta"]
    sid = meta[:, 0]
    solves = np.unique(sid)
    nval = max(1, int(len(solves) * val_frac))
    val = np.isin(sid, solves[-nval:])
    xm, xsd = x[~val].mean(0), x[~val].std(0) + 1e-12
    if norm == "global":
        ym, ysd = np.zeros(y.shape[1]), np.full(y.shape[1], y[~val].std() + 1e-12)
    else:
        ym, ysd = y[~val].mean(0), y[~val].std(0) + 1e-12
    dims = [x.shape[1], *HIDDEN, y.shape[1]]
    rng = np.random.default_rng(seed)
    layers = [(np.float32(rng.uniform(-1, 1, (a, b)) / np.sqrt(a)), np.zeros(b, np.float32))
              for a, b in zip(dims[:-1], dims[1:])]
    xs, ys, rows = (x - xm) / xsd, (y - ym) / ysd, (~val).astype(np.uint8)
    curve, t0 = [], time.time()
    for epochs, lr in schedule:
        _, layers, tl, _ = N.mlp16_train(layers, xs, ys, rows, epochs, lr, weight_decay, eval_every=eval_every)
        curve.append(tl[::max(1, epochs // 100)])
    # errors in target units (what the warm start is off by), and the ATA start's
    pred = N.mlp16_forward(layers, np.float32(xs)) * ysd + ym
    mse_val = float(((pred[val] - y[val]) ** 2).mean())
    mse_tr = float(((pred[~val] - y[~val]) ** 2).mean())
    mse_ata = float((y[val] ** 2).mean())
    save = {"nlayers": len(layers), "xmean": xm, "xstd": xsd, "ymean": ym, "ystd": ysd, "mask": z["mask"],
            "nset": int(z["nset"]), "so_split": float(z["so_split"]), "train_mse": mse_tr, "val_mse": mse_val,
            "val_mse_ata": mse_ata, "train_schedule": np.array(schedule, float),
            "train_loss_curve": np.concatenate(curve), "train_seconds": time.time() - t0, "n_rows": len(x),
            "n_solves": len(solves), "train_norm": norm}
    for i, (w, b) in enumerate(layers):
        save["w%d" % i] = np.asarray(w, np.float32)
        save["b%d" % i] = np.asarray(b, np.float32)
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    np.savez(out, **save)
    return mse_tr, mse_val, mse_ata


def report(model_path: str, nsolve: int, seed: int = 9001, precision: str = "mixed"):
    """Held-out alloy stacks (a seed the training never drew), energies cycled
    over the contour: CPA iterations, final error3 and device time from the
    ATA start and from the learned start, and the agreement of the converged
    tau.  Returns the per-solve rows."""
    from . import api
    model = Model(model_path)
    fam = model.family()
    rng = np.random.default_rng(seed)
    ctx = api.Context.for_problem(fam.base(fam.energies[0]), precision)
    rows = []
    try:
        for s in range(nsolve):
            ie = fam.energies[s % len(fam.energies)]
            ep = fam.problem(ie, fam.draw(rng))
            a = ctx.cpacoord(ep, check=False)
            ws = warm_start(ep, model, fam)
            b = ctx.cpacoord(ep, tminv=ws, check=False)
            d = float(np.linalg.norm(b["tauc"] - a["tauc"]) / np.linalg.norm(a["tauc"]))
            rows.append(dict(ie=ie, nk=ep.nk, it_ata=a["cpa_iterations"], it_mlp=b["cpa_iterations"],
                             err_ata=a["cpa_error"], err_mlp=b["cpa_error"], ms_ata=a["run_ms"], ms_mlp=b["run_ms"],
                             st=(a["status"], b["status"]), dtau=d))
    finally:
        ctx.close()
    return rows


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("gen")
    g.add_argument("--out", required=True)
    g.add_argument("--solves", type=int, default=5000)
    g.add_argument("--nset", type=int, default=6)
    g.add_argument("--so-split", type=float, default=0.03)
    g.add_argument("--max-seconds", type=float, default=1200.0)
    g.add_argument("--nctx", type=int, default=8)
    g.add_argument("--no-graphs", action="store_true")
    g.add_argument("--progress", type=int, default=50)
    t = sub.add_parser("train")
    t.add_argument("--data", required=True)
    t.add_argument("--out", default=DEFAULT_MODEL)
    t.add_argument("--schedule", default="4000:1e-3,4000:3e-4,4000:1e-4", help="epochs:lr phases")
    t.add_argument("--norm", choices=("global", "column"), default="global")
    r = sub.add_parser("report")
    r.add_argument("--model", default=DEFAULT_MODEL)
    r.add_argument("--solves", type=int, default=48)
    a = ap.parse_args()
    if a.cmd == "gen":
        n = generate(a.out, a.solves, Family(nset=a.nset, so_split=a.so_split), max_seconds=a.max_seconds,
                     nctx=a.nctx, graphs=not a.no_graphs, progress=a.progress)
        print("rows:", n)
    elif a.cmd == "train":
        sched = [(int(p.split(":")[0]), float(p.split(":")[1])) for p in a.schedule.split(",")]
        print("mse train / held out / held out of the ATA start: %.3e / %.3e / %.3e"
              % train(a.data, a.out, schedule=sched, norm=a.norm))
    else:
        rows = report(a.model, a.solves)
        ita = sum(r["it_ata"] for r in rows)
        itm = sum(r["it_mlp"] for r in rows)
        print("| E | nk | CPA it. ATA | CPA it. MLP | error3 ATA | error3 MLP | ms ATA | ms MLP | rel diff tau |")
        print("|---|---|---|---|---|---|---|---|---|")
        for x in rows:
            print("| %d | %d | %d | %d | %.1e | %.1e | %.1f | %.1f | %.1e |" % (
                x["ie"], x["nk"], x["it_ata"], x["it_mlp"], x["err_ata"], x["err_mlp"], x["ms_ata"], x["ms_mlp"],
                x["dtau"]))
        print("\ntotal CPA iterations: ATA %d, MLP %d (%.1f %%); device time ATA %.1f ms, MLP %.1f ms"
              % (ita, itm, 100.0 * itm / ita, sum(r["ms_ata"] for r in rows), sum(r["ms_mlp"] for r in rows)))


if __name__ == "__main__":
    main()
