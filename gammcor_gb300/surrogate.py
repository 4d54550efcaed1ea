"""Learned reconstruction of the AC integrand W(lambda).

The lambda quadrature (ACECORR, acfd.f:117-209) needs one ERPA solve per
Gauss-Legendre point. The surrogate solves ERPA only at the first and last
nodes of the 8-point rule (lambda ~ 0.02 and ~ 0.98), and predicts the six
interior values from those two solutions: W at both nodes, statistics of the
kept excitation energies, the active occupation spectrum, orbital-energy gaps
and the sizes of the system. That is 2 ERPA solves per energy instead of 8.

An ensemble of networks supplies the error estimate: three times the spread of
the members' energies. When the estimate is above the requested threshold the
energy falls back to the full 8-point quadrature, which reuses the two end-node
solves and the system's integrals and A+-B (kept on the device by a batch
session), so a fallback costs the exact quadrature plus the network.

Training data come from the exact path (FP64-accurate; it agrees with the plain
FP64 GPU path to ~1e-9 Eh). The networks are trained and evaluated by this
library's own kernels (api.Mlp); numpy only prepares features.
"""
from __future__ import annotations

import json
import time

import numpy as np
import torch

from . import api, synth

NGRID = 8
END = (0, NGRID - 1)
INNER = tuple(range(1, NGRID - 1))
NFEAT = 29


def gauss8():
    return api.gauleg(0.0, 1.0, NGRID)


def features(s: synth.System, w_end, st_end, ndimx: int) -> np.ndarray:
    """Fixed-length feature vector of one system (NFEAT values)."""
    occ_act = np.sort(s.occ[s.nin:s.nocc])[::-1]
    occ6 = np.zeros(6)
    occ6[:min(6, occ_act.size)] = occ_act[:6]
    f = np.asarray(s.extra.get("fock_diag", np.zeros(s.n)))
    inact_max = f[:s.nin].max() if s.nin else f[:s.nocc].min()
    act = f[s.nin:s.nocc]
    virt_min = f[s.nocc:].min() if s.n > s.nocc else f.max()
    gaps = [act.min() - inact_max, virt_min - act.max(), virt_min - inact_max]
    w0, w1 = float(w_end[0]), float(w_end[1])
    stats = []
    for st in st_end:
        stats += [st[0]] + [float(np.log(max(v, 1e-12))) for v in st[1:6]]
    sizes = [np.log(s.n), np.log(ndimx), s.nin / s.n, s.nact / 6.0]
    v = np.array([w0, w1, w0 / w1 if w1 != 0 else 0.0, np.log(abs(w1) + 1e-12)]
                 + list(occ6) + gaps + stats + sizes, dtype=np.float64)
    assert v.size == NFEAT
    return v


def shapes(count: int, seed: int, nmin=60, nmax=160):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        nin = int(rng.integers(5, min(25, n // 3) + 1))
        nact = int(rng.choice([2, 4, 6]))
        out.append(dict(n=n, nin=nin, nact=nact, rank=6 * n, seed=seed * 100003 + i))
    return out


def build_dataset(count: int, seed: int, device="cuda:0", chunk=32, nstreams=8, log=print,
                  nmin=60, nmax=160):
    """Systems, their 8-point W(lambda), exact energies and features."""
    x8, w8 = gauss8()
    X, W, E, info = [], [], [], []
    t0 = time.time()
    sh = shapes(count, seed, nmin, nmax)
    for c0 in range(0, count, chunk):
        systems = [synth.make_system_device(d["n"], d["nin"], d["nact"], d["rank"], d["seed"],
                                            device=device) for d in sh[c0:c0 + chunk]]
        batch = api.BatchInputs(systems, device=device)
        ec, _, wl, status, st = api.ac_energy_batched(batch, lambdas=x8, weights=w8,
                                                      nstreams=nstreams, omega_stats=True)
        for i, s in enumerate(systems):
            if status[i] != 0 or wl[i, END[1]] == 0.0:
                continue
            X.append(features(s, wl[i, list(END)], st[i, list(END)], batch.ndimx()[i]))
            W.append(wl[i])
            E.append(ec[i])
            info.append((s.n, s.nin, s.nact, batch.ndimx()[i]))
        log(f"dataset: {min(c0 + chunk, count)}/{count} systems, {time.time() - t0:.0f}s")
    return dict(X=np.array(X), W=np.array(W), E=np.array(E), info=np.array(info), x=x8, w=w8)


def targets(W: np.ndarray) -> np.ndarray:
    """Interior values relative to the last node: g_i = W(lambda_i) / W(lambda_8)."""
    return np.ascontiguousarray(W[:, list(INNER)] / W[:, [END[1]]])


def energy_from(W_end: np.ndarray, g: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Quadrature with exact end-node values and predicted interior ratios."""
    return (w[END[0]] * W_end[:, 0] + w[END[1]] * W_end[:, 1]
            + (g * w[list(INNER)][None, :]).sum(axis=1) * W_end[:, 1])


class Ensemble:
    def __init__(self, members: int = 4, hidden: int = 256, seed: int = 0):
        self.members = [api.Mlp(NFEAT, hidden, len(INNER), seed=seed + 17 * k)
                        for k in range(members)]
        self.xm = self.xs = self.gm = self.gs = None

    def _norm(self, X):
        return torch.tensor(np.ascontiguousarray((X - self.xm) / self.xs), dtype=torch.float32,
                            device="cuda")

    def fit(self, X, G, epochs=3000, lr=1e-3, log=print):
        self.xm, self.xs = X.mean(0), X.std(0) + 1e-9
        self.gm, self.gs = G.mean(0), G.std(0) + 1e-9
        xd = self._norm(X)
        gd = torch.tensor(np.ascontiguousarray((G - self.gm) / self.gs), dtype=torch.float32,
                          device="cuda")
        for k, net in enumerate(self.members):
            loss = None
            for ep in range(epochs):
                lr_ep = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))  # cosine schedule
                loss = net.train_step(xd, gd, max(lr_ep, 1e-6))
            log(f"member {k}: final training loss {loss:.3e}")

    def predict(self, X):
        xd = self._norm(X)
        return np.stack([net.forward(xd).cpu().numpy().astype(np.float64) * self.gs + self.gm
                         for net in self.members])  # (members, n, len(INNER))

    def save(self, path):
        np.savez_compressed(path, xm=self.xm, xs=self.xs, gm=self.gm, gs=self.gs,
                            params=np.stack([m.params().cpu().numpy() for m in self.members]))

    @classmethod
    def load(cls, path):
        d = np.load(path)
        ens = cls(members=d["params"].shape[0])
        for m, p in zip(ens.members, d["params"]):
            m.set_params(p)
        ens.xm, ens.xs, ens.gm, ens.gs = d["xm"], d["xs"], d["gm"], d["gs"]
        return ens


def estimate(ens: Ensemble, X, W_end, w):
    """Energy prediction and its error estimate (3 x spread of the members)."""
    outs = ens.predict(X)
    Es = np.stack([energy_from(W_end, g, w) for g in outs])
    return Es.mean(0), 3.0 * Es.std(0)


def evaluate(ens: Ensemble, data, thresholds=(1e-6, 1e-5, 1e-4, 1e-3)):
    x, w = data["x"], data["w"]
    W, E = data["W"], data["E"]
    W_end = W[:, list(END)]
    e_pred, e_est = estimate(ens, data["X"], W_end, w)
    err = np.abs(e_pred - E)
    # the method without the network: W linear in lambda through the last node
    g_lin = np.tile((x[list(INNER)] / x[END[1]])[None, :], (len(E), 1))
    err_lin = np.abs(energy_from(W_end, g_lin, w) - E)
    res = {"n": int(len(E)), "mae_network": float(err.mean()), "max_network": float(err.max()),
           "median_network": float(np.median(err)), "mae_without_network": float(err_lin.mean()),
           "max_without_network": float(err_lin.max()),
           "gain_mae": float(err_lin.mean() / max(err.mean(), 1e-300)),
           "estimate_covers_error": float(np.mean(e_est >= err))}
    for t in thresholds:
        acc = e_est <= t
        res[f"accept_rate@{t:g}"] = float(acc.mean())
        res[f"max_err_accepted@{t:g}"] = float(err[acc].max()) if acc.any() else 0.0
    return res


MODEL = __import__("pathlib").Path(__file__).resolve().parent / "data" / "surrogate_ensemble.npz"


def energies(batch, ens: Ensemble, threshold: float = 1e-6, nstreams: int = 8,
             precision: str = "fp64tc5", eig_emulation: bool = False,
             erpa_mode: str = "refined", eig_refine: int = 0):
    """AC-CAS energies of a batch with the surrogate: ERPA at the two end nodes
    for every system, the ensemble's prediction where its error estimate is at
    most `threshold`, and the six interior nodes where it is not. One session
    holds every system's integrals and A+-B between the two passes, so a
    rejected system costs the exact 8-point quadrature plus the network.
    Returns (energies, fallback mask, estimate, status)."""
    x8, w8 = gauss8()
    ends, inner = list(END), list(INNER)
    with api.AcSession(batch, precision=precision, erpa_mode=erpa_mode, nstreams=nstreams,
                       eig_emulation=eig_emulation, eig_refine=eig_refine) as ses:
        allidx = np.arange(len(batch.systems))
        wa, _, st, om = ses.points(allidx, x8[ends], omega_stats=True)
        nd = batch.ndimx()
        X = np.array([features(s, wa[i], om[i], nd[i]) for i, s in enumerate(batch.systems)])
        e_pred, e_est = estimate(ens, X, wa, w8)
        fb = ~(e_est <= threshold) | (st != 0)
        e = e_pred.copy()
        st = st.copy()
        if fb.any():
            idx = np.nonzero(fb)[0]
            wb, _, stb = ses.points(idx, x8[inner])
            e[idx] = wa[idx] @ w8[ends] + wb @ w8[inner]
            st[idx] = np.maximum(st[idx], stb)
    return e, fb, e_est, st


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="train and evaluate the integrand surrogate")
    ap.add_argument("--ntrain", type=int, default=256)
    ap.add_argument("--ntest", type=int, default=96)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--out", default="surrogate.npz")
    ap.add_argument("--data", default=None, help="reuse a dataset saved by an earlier run")
    ap.add_argument("--seed", type=int, default=77)
    a = ap.parse_args(argv)
    data_path = a.data or a.out.replace(".npz", "_data.npz")
    if a.data:
        d = np.load(a.data)
        tr = {k[3:]: d[k] for k in d.files if k.startswith("tr_")}
        te = {k[3:]: d[k] for k in d.files if k.startswith("te_")}
    else:
        tr = build_dataset(a.ntrain, a.seed)
        te = build_dataset(a.ntest, a.seed + 1)
        np.savez_compressed(data_path, **{f"tr_{k}": v for k, v in tr.items()},
                            **{f"te_{k}": v for k, v in te.items()})
    ens = Ensemble(members=a.members)
    t0 = time.time()
    ens.fit(tr["X"], targets(tr["W"]), epochs=a.epochs)
    train_s = time.time() - t0
    ens.save(a.out)
    res = {"train": evaluate(ens, tr), "test": evaluate(ens, te), "train_seconds": train_s,
           "ntrain": int(len(tr["E"])), "ntest": int(len(te["E"]))}
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
