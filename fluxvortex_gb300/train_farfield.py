"""Trains the learned far-field operator and writes its weights.

    python -m fluxvortex_gb300.train_farfield [--out fluxvortex_gb300/data/farfield_mlp.npz]

Training pairs come from the solver's own particle fields, swept by the
treecode with every accepted (target leaf, source cell) pair on the
local-expansion path and sampled with FP64 direct-sum targets; the network
fits the residual of the analytic multipole-to-local translation, each pair
weighted by 1/|T|^2 so that the relative error of every expansion counts:
  * the synthetic slab wake (particles uniform in a 20c x 10c x 2c slab,
    strengths i.i.d. normal, sigma = 0.02c) at several sizes and seeds;
  * the heaving-wing hybrid run (panel wing shedding ring rows that are
    converted to particles, seeded with a slab wake) after some steps, when
    the converted sheet and the self-advected slab have formed.
Several leaf sizes give the network the range of h_T / d and h_S / d the
sweeps see.  A separate seed forms the validation set; its per-pair error
statistics are stored with the weights.
"""
from __future__ import annotations

import argparse
import time

import numpy as np
import torch

from . import learned as L
from .tree import TreeSweeper
from .workloads import slab_wake


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def slab_fields(sizes, seeds):
    for n in sizes:
        for s in seeds:
            pos, gam, sig, _ = slab_wake(n, seed=s)
            yield f"slab n={n} seed={s}", _dev(pos), _dev(gam), _dev(sig), n


def hybrid_field(n_seed, steps, seed):
    from .geometry import heaving_wing
    from .hybrid import HybridStep
    pos, gam, sig, _ = slab_wake(n_seed, seed=seed)
    cfg = heaving_wing(n_keep=10, free_vpm=True, stretch=True, rlxf=0.0,
                       max_particles=n_seed + 48 * (steps + 8), far_field="tree")
    hs = HybridStep(cfg, precision="f32c", device="cuda")
    hs.field.add_particles_batch(pos, gam, sig)
    for _ in range(steps):
        hs.step()
    f = hs.field
    n = f.np
    return (f"hybrid n={n} steps={steps} seed={seed}", f._pos[:n].clone(), f._gamma[:n].clone(),
            f._sigma[:n].clone(), n)


def collect(fields, per_field, leaves, log=print, theta=0.5):
    Xs, Ts, As = [], [], []
    for name, pos, gam, sig, n in fields:
        for leaf in leaves:
            ts = TreeSweeper(theta=theta, leaf_target=leaf)
            X, T, A = L.harvest(ts, pos, gam, sig, n, per_field)
            Xs.append(X)
            Ts.append(T)
            As.append(A)
            log(f"  {name} leaf={leaf}: {X.shape[0]} pairs")
    return torch.cat(Xs), torch.cat(Ts), torch.cat(As)


def _stats(e):
    e = e.cpu().numpy()
    return {"median": float(np.median(e)), "p90": float(np.percentile(e, 90)),
            "p99": float(np.percentile(e, 99)), "max": float(e.max())}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--out", default=L.DEFAULT_WEIGHTS)
    p.add_argument("--steps", type=int, default=8000)
    p.add_argument("--batch", type=int, default=8192)
    p.add_argument("--lr", type=float, default=2e-3)
    p.add_argument("--per-field", type=int, default=65536)
    p.add_argument("--hybrid-steps", type=int, default=6)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--quick", action="store_true", help="small data and few steps")
    p.add_argument("--theta", type=float, default=0.5,
                   help="opening angle of the treecode whose accepted pairs are trained on")
    a = p.parse_args(argv)
    t0 = time.time()
    sizes = (1 << 14, 1 << 16) if a.quick else (1 << 16, 1 << 18, 1 << 20)
    leaves = (32, 64) if a.quick else (16, 32, 64)
    train = list(slab_fields(sizes, (101, 102)))
    train.append(hybrid_field(sizes[-1] // 4, a.hybrid_steps, 103))
    print("training fields:")
    X, T, A = collect(train, a.per_field, leaves, theta=a.theta)
    del train
    print("validation fields:")
    Xv, Tv, Av = collect(list(slab_fields(sizes[-1:], (201,))) +
                     [hybrid_field(sizes[-1] // 4, a.hybrid_steps, 202)],
                     a.per_field // 2, leaves, theta=a.theta)
    print(f"{X.shape[0]} training / {Xv.shape[0]} validation pairs ({time.time() - t0:.1f} s)")
    m = L.FarFieldMLP(seed=a.seed)
    steps = 300 if a.quick else a.steps
    hist = m.fit(X, T - A, steps=steps, batch=a.batch, lr=a.lr, seed=a.seed,
                 log_every=max(1, steps // 10), weights=L.relative_weights(T))
    for it, loss in hist:
        print(f"  step {it:6d}  residual mse {loss:.3e}")
    tr, va = _stats(m.errors(X, T, A)), _stats(m.errors(Xv, Tv, Av))
    an = _stats(L.analytic_errors(Tv, Av))
    print("train relative error (analytic + learned)", tr)
    print("validation relative error (analytic + learned)", va)
    print("validation relative error (analytic alone)", an)
    m.save(a.out, n_train=X.shape[0], steps=steps, batch=a.batch, lr=a.lr, theta=a.theta,
           val_median=va["median"], val_p90=va["p90"], val_p99=va["p99"], val_max=va["max"],
           val_analytic_median=an["median"], val_analytic_p90=an["p90"],
           val_analytic_p99=an["p99"], train_median=tr["median"])
    print(f"wrote {a.out} ({time.time() - t0:.1f} s)")


if __name__ == "__main__":
    main()
