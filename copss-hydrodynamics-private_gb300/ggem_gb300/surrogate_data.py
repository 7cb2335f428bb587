"""Training set and training run of the eigen-interval network.

Configurations follow the learned-surrogate workload: N log-uniform in
[1000, 50000] beads of radius 1 (the shipped network: [1000, 200000], so
that the benchmark's 200k-bead suspension lies inside the training range),
volume fraction uniform in [0.02, 0.2],
a chain fraction from {0, 1/4, 1/2, 3/4, 1} of the beads in 20-bead chains
(bond 2a, self-avoiding growth) and the rest free (random sequential
addition), periodic cube, alpha = 0.5, rc = 7.  Each configuration gives
the features of ggem_surrogate_features (computed on the GPU from the FP32
pair list) and the labels log lambda_min, log lambda_max of the local
mobility from the library's Lanczos (FP64 recurrence with full
reorthogonalisation over the FP32 pair-sum operator).

The network is trained on the GPU by the library's own tensor-core forward
and backward kernels (ggem_surrogate_train).  The safety margins that widen
a prediction are multiples of the held-out RMSE of each log-bound.

Command line (writes an .npz with the parameters, the normalisation, the
margins and the held-out statistics):

    python -m ggem_gb300.surrogate_data --configs 22000 --holdout 2000 \
        --n-max 200000 --out eigen_surrogate.npz
"""
from __future__ import annotations

import argparse
import json
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

from . import FP32, SUR_FEATURES, Context, Surrogate, make_mixture

BEADS_PER_CHAIN = 20
CHAIN_FRACTIONS = (0.0, 0.25, 0.5, 0.75, 1.0)
ALPHA, RC = 0.5, 7.0


def sample_configs(count, seed, n_range=(1000, 50000), phi_range=(0.02, 0.2)):
    """Seeded configuration descriptions (no positions yet)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        phi = float(rng.uniform(*phi_range))
        cf = CHAIN_FRACTIONS[int(rng.integers(len(CHAIN_FRACTIONS)))]
        n_chains = int(round(cf * n / BEADS_PER_CHAIN))
        n_free = max(n - BEADS_PER_CHAIN * n_chains, 0)
        if n_chains == 0 and n_free == 0:
            n_free = n
        total = BEADS_PER_CHAIN * n_chains + n_free
        out.append({"seed": int(seed) * 1_000_003 + k, "n_chains": n_chains, "n_free": n_free,
                    "phi": phi, "chain_fraction": BEADS_PER_CHAIN * n_chains / total})
    return out


def range_kwargs(summary):
    """the bead-count and volume-fraction ranges of a training run (the
    summary of save()), as keyword arguments of sample_configs"""
    return {"n_range": tuple(summary.get("n_range", (1000, 50000))),
            "phi_range": tuple(summary.get("phi_range", (0.02, 0.2)))}


def positions(cfg):
    return make_mixture(cfg["seed"], cfg["n_chains"], BEADS_PER_CHAIN, cfg["n_free"], 2.0,
                        cfg["phi"])


def label(cfgs, k=60, device=0, threads=16, chunk=64, log=None):
    """Features X [n x 35] and labels Y [n x 2] (log lambda_min, log lambda_max);
    positions are generated on host threads a chunk ahead of the GPU work."""
    X = np.zeros((len(cfgs), SUR_FEATURES), np.float32)
    Y = np.zeros((len(cfgs), 2), np.float32)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        pending = ex.map(positions, cfgs[:chunk])
        for c0 in range(0, len(cfgs), chunk):
            batch = list(pending)
            nxt = cfgs[c0 + chunk:c0 + 2 * chunk]
            pending = ex.map(positions, nxt)
            for j, (xyz, L) in enumerate(batch):
                i = c0 + j
                with Context(alpha=ALPHA, box_hi=(L,) * 3, rc=RC, precision=FP32,
                             device=device) as ctx:
                    ctx.set_particles(xyz)
                    ctx.build_cells()
                    X[i] = ctx.surrogate_features(cfgs[i]["chain_fraction"])
                    lo, hi = ctx.lanczos_bounds(k=k, seed=1)
                    Y[i] = (np.log(lo), np.log(hi))
            if log and (c0 // chunk) % 20 == 0:
                log(f"labelled {min(c0 + chunk, len(cfgs))}/{len(cfgs)} "
                    f"in {time.perf_counter() - t0:.1f} s")
    return X, Y


def train(X, Y, Xh, Yh, epochs=300, batch=256, lr=2e-3, seed=0, device=0, sigmas=3.0):
    """Train on (X, Y), evaluate on the held-out (Xh, Yh); returns the network
    and a summary with the margins (sigmas x held-out RMSE per log-bound)."""
    sur = Surrogate(device=device, seed=seed + 1)
    sur.fit_norm(X, Y)
    t0 = time.perf_counter()
    loss = sur.train(X, Y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    t_train = time.perf_counter() - t0
    P = sur.predict(Xh)
    err = P - Yh
    rmse = np.sqrt((err ** 2).mean(axis=0))
    margins = sigmas * rmse
    cover = float(np.mean((P[:, 0] - margins[0] <= Yh[:, 0]) & (P[:, 1] + margins[1] >= Yh[:, 1])))
    summary = {"epochs": epochs, "batch": batch, "lr": lr, "train_seconds": t_train,
               "loss_first": float(loss[0]), "loss_last": float(loss[-1]),
               "holdout_rmse_log": rmse.tolist(), "holdout_max_abs_log": np.abs(err).max(0).tolist(),
               "margins_log": margins.tolist(), "holdout_coverage": cover,
               "n_train": int(len(X)), "n_holdout": int(len(Xh))}
    return sur, summary, loss


def save(path, sur, summary, loss):
    np.savez(path, params=sur.params, norm=sur.norm,
             margins=np.asarray(summary["margins_log"], np.float64), loss=loss,
             summary=json.dumps(summary))


DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "data" / "eigen_surrogate.npz"


def load_default(device=0):
    """The network trained by this module's command line on 20000 + 2000
    configurations (None when the file is absent)."""
    if not DEFAULT_WEIGHTS.exists():
        return None
    return load(DEFAULT_WEIGHTS, device=device)


def load(path, device=0):
    """(network, margins, summary) from a file written by save()."""
    d = np.load(path, allow_pickle=False)
    sur = Surrogate(device=device)
    sur.norm = d["norm"]
    sur.params = d["params"]
    return sur, d["margins"], json.loads(str(d["summary"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", type=int, default=22000)
    ap.add_argument("--holdout", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--lanczos-k", type=int, default=60)
    ap.add_argument("--n-min", type=int, default=1000)
    ap.add_argument("--n-max", type=int, default=50000)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", required=True)
    ap.add_argument("--data-out", default=None, help="also save X, Y")
    a = ap.parse_args()
    from .build import build
    build()
    n_range = (a.n_min, a.n_max)
    cfgs = sample_configs(a.configs, a.seed, n_range=n_range)
    t0 = time.perf_counter()
    X, Y = label(cfgs, k=a.lanczos_k, log=lambda m: print(m, flush=True))
    t_label = time.perf_counter() - t0
    ntr = a.configs - a.holdout
    sur, summary, loss = train(X[:ntr], Y[:ntr], X[ntr:], Y[ntr:], epochs=a.epochs,
                               batch=a.batch, lr=a.lr, seed=a.seed)
    summary.update({"label_seconds": t_label, "lanczos_k": a.lanczos_k, "configs": a.configs,
                    "seed": a.seed, "n_range": list(n_range), "phi_range": [0.02, 0.2]})
    save(a.out, sur, summary, loss)
    if a.data_out:
        np.savez(a.data_out, X=X, Y=Y)
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
