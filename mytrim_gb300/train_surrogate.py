"""Train the scattering surrogate on the GPU and store its parameters.

    python -m mytrim_gb300.train_surrogate [--target magic|quadrature]
                                           [--weighting transfer|uniform] [--epochs 24]

Trains the MLP 2 -> 64 -> 64 -> 64 -> 2 on 2e7 samples (log-uniform reduced energy
in [1e-4, 1e4], area-weighted reduced impact parameter in [0, 12]) with the
engine's own kernels (mtg_surrogate_train).  Each sample's time integral comes from
FP64 Gauss-Mehler quadrature; its sin^2(theta/2) target is either

* the FP64 magic formula (trim.C:180-271) at the sample -- the network the
  surrogate path runs by default (surrogate_params.npy): the plain path and the
  FP64 oracle evaluate that formula, and the surrogate is judged against them; or
* the quadrature itself (surrogate_params_quadrature.npy): the true scattering
  integral, which the magic formula approximates to about 1 %.

It writes the parameters (8642 float32) and a JSON report beside them: the
network's error against both targets on held-out points of the domain where it
runs (eps <= 10), and the energy-transfer-weighted signed bias per decade of eps.
"""
import argparse
import json
import time
from pathlib import Path

import numpy as np

from .engine import Engine

DATA = Path(__file__).resolve().parent / "data"
PARAMS = DATA / "surrogate_params.npy"                       # magic-formula target (default)
PARAMS_QUADRATURE = DATA / "surrogate_params_quadrature.npy"  # quadrature target
REPORT = DATA / "surrogate_eval.json"
REPORT_QUADRATURE = DATA / "surrogate_eval_quadrature.json"
EPS_NET_MAX = 10.0  # the network stands in for the magic formula up to here (mtg_surrogate.cuh)


def evaluate(e, n=400_000, seed=12345):
    """Errors of the context's network on held-out points where it runs."""
    rng = np.random.default_rng(seed)
    eps = 10 ** rng.uniform(-4, np.log10(EPS_NET_MAX), n)
    b = 12 * np.sqrt(rng.uniform(0, 1, n))
    s2q, _ = e.quadrature(eps, b)
    s2n = e.scatter(eps, b, precision="surrogate")
    s2m = e.scatter(eps, b, precision="fp64")
    le = np.log10(eps)
    out = {"points": n, "domain": "log10 eps in [-4, 1], b in [0, 12] area-weighted"}
    for name, s2, ref in (("network_vs_quadrature", s2n, s2q), ("network_vs_magic", s2n, s2m),
                          ("magic_vs_quadrature", s2m, s2q)):
        rel = np.abs(s2 - ref) / np.maximum(ref, 1e-300)
        m = ref > 1e-4
        out[f"{name}_median_rel"] = float(np.median(rel[m]))
        out[f"{name}_p95_rel"] = float(np.quantile(rel[m], 0.95))
        # energy transfer and angular diffusion go with s2: the signed error weighted by it
        out[f"{name}_transfer_bias_per_decade"] = [
            float(np.sum((s2 - ref)[(le >= lo) & (le < lo + 1)]) / np.sum(ref[(le >= lo) & (le < lo + 1)]))
            for lo in range(-4, 1)]
        out[f"{name}_transfer_abs_rel"] = float(np.sum(np.abs(s2 - ref)) / np.sum(ref))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=20_000_000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--epochs", type=int, default=24)
    ap.add_argument("--qat-epochs", type=int, default=2)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--target", default="magic", choices=["magic", "quadrature"],
                    help="sin^2(theta/2) target: the magic formula, or the quadrature at the same samples")
    ap.add_argument("--weighting", default="transfer", choices=["transfer", "uniform"],
                    help="loss weight per sample: its sin^2(theta/2) (transfer) or 1 (uniform)")
    ap.add_argument("--out", default=None, help="parameter file (default: by target, in mytrim_gb300/data)")
    a = ap.parse_args()
    out = Path(a.out) if a.out else (PARAMS if a.target == "magic" else PARAMS_QUADRATURE)
    report = out.with_name(out.stem.replace("surrogate_params", "surrogate_eval") + ".json")
    e = Engine(precision="fp32")
    t0 = time.time()
    rep = e.surrogate_train(n_train=a.n_train, batch=a.batch, epochs=a.epochs, qat_epochs=a.qat_epochs, lr=a.lr,
                            seed=a.seed, target=a.target, weighting=a.weighting)
    wall = time.time() - t0
    np.save(out, e.surrogate_params())
    ev = evaluate(e)
    ev.update({"train": rep, "wall_seconds": wall, "config": {**vars(a), "out": out.name}})
    report.write_text(json.dumps(ev, indent=1))
    print(json.dumps(ev))
    e.close()


if __name__ == "__main__":
    main()
