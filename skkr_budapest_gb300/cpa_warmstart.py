"""Learned warm start of the CPA loop.

The CPA iteration of rsp-scf/fullcpa.f (cpacor/cpasol) starts from the
coherent inverse t-matrix m_c it is given: the ATA average (tata,
fullcpa.f:2-23) or an effective t-matrix read back from a previous run
(main/tcpaio.f:193-276).  Here a small MLP maps the single-site data of one
alloy layer at one energy to its converged m_c; the CPA iteration itself is
unchanged (same update, same error3 test, same tolerance), only its starting
point moves, so the converged result is the same up to the CPA tolerance.

Features of (alloy layer, energy), from the (kappa,mu)-diagonal screened
inverse t-matrices of the two species (one value per kappa):
    Re E, Im E, c, Re/Im m_A(kappa), Re/Im m_B(kappa)
Target, per kappa: (m_c(kappa) - m_ATA(kappa)) / |m_A(kappa) - m_B(kappa)|
(Re, Im), with m_c(kappa) the mu-average of the converged diagonal.  The
warm start is m_ATA + diag(prediction), off-diagonal elements from ATA (zero
for these diagonal species).  The "continuation" variant also reads the
converged target of the same layer at the previous contour energy (a proxy
for the lattice environment, which the single-site features cannot see).

    python -m skkr_budapest_gb300.cpa_warmstart gen   --out data.npz     (GPU)
    python -m skkr_budapest_gb300.cpa_warmstart train --data data.npz --out model.npz
    python -m skkr_budapest_gb300.cpa_warmstart report --model model.npz    (GPU)
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

from . import synth as S
from . import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "data", "cpa_mlp_bcc_lmax3.npz")


def kappa_groups(lmax: int):
    """Index arrays of the (kappa,mu) basis grouped by kappa (clebsch.f order)."""
    _, kv = S.kmy_l_kappa(lmax)
    kappas = []
    for k in kv.tolist():
        if k not in kappas:
            kappas.append(k)
    return [np.nonzero(kv == k)[0] for k in kappas]


def _kdiag(m: np.ndarray, groups) -> np.ndarray:
    d = np.diag(m)
    return np.array([d[g].mean() for g in groups])


def layer_features(ep, li: int, groups) -> np.ndarray:
    ma = _kdiag(ep.tminva[li], groups)
    mb = _kdiag(ep.tminvb[li], groups)
    return np.concatenate([[ep.ce.real, ep.ce.imag, ep.conc[li]], ma.real, ma.imag, mb.real, mb.imag])


def _ata_kdiag(ep, li, groups):
    ma = _kdiag(ep.tminva[li], groups)
    mb = _kdiag(ep.tminvb[li], groups)
    c = ep.conc[li]
    ata = ma * mb / (c * mb + (1.0 - c) * ma)   # tata for diagonal species
    return ata, np.abs(ma - mb) + 1e-30


def layer_target(ep, li: int, mc: np.ndarray, groups) -> np.ndarray:
    ata, scale = _ata_kdiag(ep, li, groups)
    r = (_kdiag(mc, groups) - ata) / scale
    return np.concatenate([r.real, r.imag])


class Model:
    """Inference of the trained MLP (tanh hidden layers) in numpy."""

    def __init__(self, path: str = DEFAULT_MODEL):
        z = np.load(path)
        self.layers = [(z["w%d" % i], z["b%d" % i]) for i in range(int(z["nlayers"]))]
        self.xmean, self.xstd = z["xmean"], z["xstd"]
        self.ymean, self.ystd = z["ymean"], z["ystd"]
        self.lmax = int(z["lmax"])
        self.cont = bool(z["cont"]) if "cont" in z else False

    def predict(self, x: np.ndarray, device: str = "cpu") -> np.ndarray:
        h = (np.atleast_2d(x) - self.xmean) / self.xstd
        if device == "gpu":
            from . import native as N
            return N.mlp_forward(self.layers, h) * self.ystd + self.ymean
        for i, (w, b) in enumerate(self.layers):
            h = h @ w + b
            if i < len(self.layers) - 1:
                h = np.tanh(h)
        return h * self.ystd + self.ymean


def warm_start(ep, model: Model, prev=None) -> np.ndarray:
    """Starting coherent t^-1 for every interface layer: the MLP estimate on
    alloy layers (conc strictly between 0 and 1), the given one elsewhere.
    prev = (EnergyProblem, converged tminv) of the previous contour energy,
    read by a continuation model (zeros without it)."""
    groups = kappa_groups(ep.lmax)
    tm = np.array(ep.tminv, copy=True)
    alloy = [li for li in range(ep.nintfc) if 1e-6 < ep.conc[li] < 1.0 - 1e-6]
    if not alloy:
        return tm
    feats = []
    for li in alloy:
        f = layer_features(ep, li, groups)
        if model.cont:
            pt = (layer_target(prev[0], li, prev[1][li], groups) if prev is not None
                  else np.zeros(2 * len(groups)))
            f = np.concatenate([f, pt])
        feats.append(f)
    pred = model.predict(np.array(feats))
    ng = len(groups)
    for row, li in zip(pred, alloy):
        ata, scale = _ata_kdiag(ep, li, groups)
        mk = ata + (row[:ng] + 1j * row[ng:]) * scale
        m = np.zeros_like(tm[li])
        for g, v in zip(groups, mk):
            m[g, g] = v
        tm[li] = m
    return tm


def _spec(seed: int, lmax: int = 3):
    # the committed models were trained on the j-split (0.03 Ry) inputs
    spec = W.rel_bcc_cpa(nsets=[4] * 24, so_split=0.03)
    spec.seed = seed
    spec.lmax = lmax
    return spec


def generate(out: str, seeds, nset: int, lmax: int = 3, max_seconds: float = 1e9, precision="fp64"):
    """Converged CPA solutions of seeded C4 variants (4 alloy layers each) on
    nset meshes, all 24 contour energies: (features, targets) per alloy layer."""
    from . import api
    groups = kappa_groups(lmax)
    xs, ys, meta = [], [], []
    t0 = time.time()
    ctx = None
    for seed in seeds:
        spec = _spec(seed, lmax)
        for ie in range(len(spec.energies)):
            ep = W.energy_problem(spec, ie, nset=nset)
            if ctx is None:
                ctx = api.Context.for_problem(ep, precision)
            r = ctx.cpacoord(ep, check=False)
            if r["status"] != 0:
                continue
            for li in spec.alloy_layers:
                xs.append(layer_features(ep, li, groups))
                ys.append(layer_target(ep, li, r["tminv"][li], groups))
                meta.append((seed, ie, li, r["cpa_iterations"]))
        print("seed %d: %d samples, %.1f s" % (seed, len(xs), time.time() - t0), flush=True)
        if time.time() - t0 > max_seconds:
            break
    ctx.close()
    np.savez(out, x=np.array(xs), y=np.array(ys), meta=np.array(meta), lmax=lmax, nset=nset)
    return len(xs)


def _dataset(data: str, cont: bool, itcpam: int = 50):
    """(x, y, seed) of the converged samples; cont appends the previous
    energy's target of the same (seed, layer) (samples without one dropped)."""
    z = np.load(data)
    x, y, meta = z["x"], z["y"], z["meta"]
    ok = meta[:, 3] < itcpam                      # CPA converged within its cap
    if cont:
        key = {(int(a), int(b), int(c)): i for i, (a, b, c, _) in enumerate(meta)}
        prev = np.array([key.get((int(a), int(b) - 1, int(c)), -1) for a, b, c, _ in meta])
        ok &= prev >= 0
        ok &= meta[np.maximum(prev, 0), 3] < itcpam
        x = np.c_[x, y[np.maximum(prev, 0)]]
    return x[ok], y[ok], meta[ok, 0], int(z["lmax"])


def train(data: str, out: str, hidden: int = 64, epochs: int = 3000, seed: int = 0, val_frac: float = 0.1,
          cont: bool = False, weight_decay: float = 1e-4, device: str = "cpu"):
    """Full-batch AdamW on the mean squared error of the targets (one global
    target scale); the last val_frac of the seeds is held out and the epoch
    with the lowest held-out error is kept.  device "gpu": this library's
    forward, backward and AdamW kernels (skkr_gpu_mlp_train) from a seeded
    uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) start; "cpu": torch."""
    x, y, sd, lmax = _dataset(data, cont)
    seeds = np.unique(sd)
    nval = max(1, int(len(seeds) * val_frac))
    val = np.isin(sd, seeds[-nval:])
    xm, xsd = x[~val].mean(0), x[~val].std(0) + 1e-12
    ym, ysd = np.zeros(y.shape[1]), np.full(y.shape[1], y[~val].std() + 1e-12)
    dims = [x.shape[1], hidden, hidden, y.shape[1]]
    if device == "gpu":
        from . import native as N
        rng = np.random.default_rng(seed)
        init = [(rng.uniform(-1, 1, (a, b)) / np.sqrt(a), rng.uniform(-1, 1, b) / np.sqrt(a))
                for a, b in zip(dims[:-1], dims[1:])]
        _, wts, _, (vl, tl) = N.mlp_train(init, (x - xm) / xsd, (y - ym) / ysd, (~val).astype(np.uint8),
                                          epochs, 2e-3, weight_decay, eval_every=20)
        return _save_model(out, wts, xm, xsd, ym, ysd, lmax, cont, tl, vl, y, val)
    import torch
    torch.manual_seed(seed)
    lins = [torch.nn.Linear(a, b, dtype=torch.float64) for a, b in zip(dims[:-1], dims[1:])]
    params = [p for l in lins for p in l.parameters()]
    opt = torch.optim.AdamW(params, lr=2e-3, weight_decay=weight_decay)

    def fwd(t):
        for i, l in enumerate(lins):
            t = l(t)
            if i < len(lins) - 1:
                t = torch.tanh(t)
        return t

    xt = torch.tensor((x - xm) / xsd)
    yt = torch.tensor((y - ym) / ysd)
    tr = torch.tensor(~val)
    best = (float("inf"), None, None)
    for ep_ in range(epochs):
        opt.zero_grad()
        loss = ((fwd(xt[tr]) - yt[tr]) ** 2).mean()
        loss.backward()
        opt.step()
        if ep_ % 20 == 0 or ep_ == epochs - 1:
            with torch.no_grad():
                vl = ((fwd(xt[~tr]) - yt[~tr]) ** 2).mean().item()
            if vl < best[0]:
                best = (vl, loss.item(), [(l.weight.detach().clone(), l.bias.detach().clone()) for l in lins])
    vl, tl, wts = best
    wts = [(w.numpy().T.copy(), b.numpy().copy()) for w, b in wts]
    return _save_model(out, wts, xm, xsd, ym, ysd, lmax, cont, tl, vl, y, val)


def _save_model(out, wts, xm, xsd, ym, ysd, lmax, cont, tl, vl, y, val):
    save = {"nlayers": len(wts), "xmean": xm, "xstd": xsd, "ymean": ym, "ystd": ysd, "lmax": lmax,
            "cont": int(cont), "train_mse": tl * ysd[0] ** 2, "val_mse": vl * ysd[0] ** 2,
            "val_mse_ata": float((y[val] ** 2).mean())}
    for i, (w, b) in enumerate(wts):
        save["w%d" % i] = np.asarray(w, np.float64)
        save["b%d" % i] = np.asarray(b, np.float64)
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    np.savez(out, **save)
    return save["train_mse"], save["val_mse"], save["val_mse_ata"]


def report(model_paths, seeds, energies, nset: int, lmax: int = 3, precision="fp64"):
    """CPA iterations, final error3 and device time from the ATA start and
    from each learned start on held-out configurations, energies in contour
    order (a continuation model reads its own previous converged result),
    and the agreement of the converged tau with the ATA-started run."""
    from . import api
    models = [Model(p) for p in model_paths]
    rows = []
    for seed in seeds:
        spec = _spec(seed, lmax)
        prev = [None] * len(models)
        ctx = None
        for ie in energies:
            ep = W.energy_problem(spec, ie, nset=nset)
            if ctx is None:
                ctx = api.Context.for_problem(ep, precision)
            a = ctx.cpacoord(ep, check=False)
            row = dict(seed=seed, ie=ie, nk=ep.nk, runs=[("ATA", a["cpa_iterations"], a["cpa_error"], a["run_ms"], 0.0,
                                                            a["status"])])
            for i, (mp, model) in enumerate(zip(model_paths, models)):
                b = ctx.cpacoord(ep, tminv=warm_start(ep, model, prev[i]), check=False)
                d = np.linalg.norm(b["tauc"] - a["tauc"]) / np.linalg.norm(a["tauc"])
                row["runs"].append((os.path.basename(mp), b["cpa_iterations"], b["cpa_error"], b["run_ms"], d,
                                    b["status"]))
                prev[i] = (ep, b["tminv"]) if b["status"] == 0 else None
            rows.append(row)
        ctx.close()
    return rows


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("gen")
    g.add_argument("--out", required=True)
    g.add_argument("--seeds", type=int, default=200)
    g.add_argument("--seed0", type=int, default=1000)
    g.add_argument("--nset", type=int, default=4)
    g.add_argument("--max-seconds", type=float, default=600.0)
    t = sub.add_parser("train")
    t.add_argument("--data", required=True)
    t.add_argument("--out", default=DEFAULT_MODEL)
    t.add_argument("--epochs", type=int, default=3000)
    t.add_argument("--cont", action="store_true")
    t.add_argument("--device", choices=("cpu", "gpu"), default="cpu")
    r = sub.add_parser("report")
    r.add_argument("--models", default=DEFAULT_MODEL)
    r.add_argument("--seeds", default="9001,9002,9003")
    r.add_argument("--energies", default="0,2,4,6,8,10,12,14,16")
    r.add_argument("--nset", type=int, default=20)
    a = ap.parse_args()
    if a.cmd == "gen":
        n = generate(a.out, range(a.seed0, a.seed0 + a.seeds), a.nset, max_seconds=a.max_seconds)
        print("samples:", n)
    elif a.cmd == "train":
        print("mse train / held out / held out of the ATA start: %.3e / %.3e / %.3e" % train(
            a.data, a.out, epochs=a.epochs, cont=a.cont, device=a.device))
    else:
        paths = a.models.split(",")
        rows = report(paths, [int(s) for s in a.seeds.split(",")], [int(e) for e in a.energies.split(",")],
                      a.nset)
        names = [r[0] for r in rows[0]["runs"]]
        print("| seed | E | nk | " + " | ".join("CPA it. %s | error3 %s | ms %s" % (n, n, n) for n in names)
              + " | max rel diff tau |")
        print("|---|---|---|" + "---|---|---|" * len(names) + "---|")
        tot = np.zeros(len(names))
        ms = np.zeros(len(names))
        for x in rows:
            cells = []
            for k, (n, it, er, t, d, st) in enumerate(x["runs"]):
                cells.append("%d | %.1e | %.1f" % (it, er, t))
                tot[k] += it
                ms[k] += t
            print("| %d | %d | %d | %s | %.1e |" % (x["seed"], x["ie"], x["nk"], " | ".join(cells),
                                                   max(r[4] for r in x["runs"])))
        print()
        for n, it, t in zip(names, tot, ms):
            print("%s: %d CPA iterations (%.1f%% of ATA), %.1f ms device time" % (n, it, 100 * it / tot[0], t))


if __name__ == "__main__":
    main()
