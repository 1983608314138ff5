"""Train the scattering surrogate on the GPU and store its parameters.

    python -m mytrim_gb300.train_surrogate [--n-train 20000000] [--epochs 12]

Trains the MLP 2 -> 64 -> 64 -> 64 -> 2 on FP64 Gauss-Mehler quadrature samples
with the engine's own kernels (mtg_surrogate_train), then writes
mytrim_gb300/data/surrogate_params.npy (8642 float32) and surrogate_eval.json:
the network's and the magic formula's error against the quadrature on held-out
points, which is what the surrogate gains over the method without it.
"""
import argparse
import json
import time
from pathlib import Path

import numpy as np

from .engine import Engine

DATA = Path(__file__).resolve().parent / "data"
PARAMS = DATA / "surrogate_params.npy"
REPORT = DATA / "surrogate_eval.json"


def evaluate(e, n=200_000, seed=12345):
    rng = np.random.default_rng(seed)
    eps = 10 ** rng.uniform(-4, 4, n)
    b = 12 * np.sqrt(rng.uniform(0, 1, n))
    s2q, _ = e.quadrature(eps, b)
    s2n = e.scatter(eps, b, precision="surrogate")
    s2m = e.scatter(eps, b, precision="fp64")
    out = {}
    for name, s2 in (("network", s2n), ("exact_path", s2m)):
        rel = np.abs(s2 - s2q) / np.maximum(s2q, 1e-300)
        for lo, tag in ((1e-4, "s2>1e-4"), (1e-8, "s2>1e-8")):
            m = s2q > lo
            out[f"{name}_{tag}_median_rel"] = float(np.median(rel[m]))
            out[f"{name}_{tag}_p95_rel"] = float(np.quantile(rel[m], 0.95))
        # energy-transfer-weighted error: sum |s2 - s2q| b db over sum s2q b db
        out[f"{name}_transfer_weighted_rel"] = float(np.sum(np.abs(s2 - s2q)) / np.sum(s2q))
    low = eps <= 10
    out["exact_path_uses_magic_formula_for_eps<=10"] = True
    rel_m = np.abs(s2m[low] - s2q[low]) / s2q[low]
    rel_n = np.abs(s2n[low] - s2q[low]) / s2q[low]
    out["eps<=10_median_rel_network"] = float(np.median(rel_n))
    out["eps<=10_median_rel_magic"] = float(np.median(rel_m))
    out["points"] = n
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=20_000_000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--qat-epochs", type=int, default=2)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=str(PARAMS))
    a = ap.parse_args()
    e = Engine(precision="fp32")
    t0 = time.time()
    rep = e.surrogate_train(n_train=a.n_train, batch=a.batch, epochs=a.epochs, qat_epochs=a.qat_epochs, lr=a.lr,
                            seed=a.seed)
    wall = time.time() - t0
    p = e.surrogate_params()
    np.save(a.out, p)
    ev = evaluate(e)
    ev.update({"train": rep, "wall_seconds": wall, "config": vars(a)})
    Path(a.out).with_name(REPORT.name).write_text(json.dumps(ev, indent=1))
    print(json.dumps(ev))
    e.close()


if __name__ == "__main__":
    main()
