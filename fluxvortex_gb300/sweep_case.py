"""One treecode self-sweep pair (velocity, then stretching) of the seeded slab wake.

    python -m fluxvortex_gb300.sweep_case [--n 1048576] [--leaf 48] [--far-field learned]
        [--repeat 0]

The smallest complete invocation of the particle hot path: the slab wake of
``workloads.slab_wake`` (uniform in a 20c x 10c x 2c slab, sigma 0.02c),
one velocity and one stretching sweep with the chosen far field, FP64
validation off.  Used as the profiling case of the evaluation and network
kernels (and handy to time one sweep of a given size: ``--repeat R`` runs R
more sweep pairs at the same positions and prints the median times of the
evaluation kernel and of the local-expansion stage, from CUDA events).
"""
from __future__ import annotations

import argparse

import torch

from . import _capi
from .tree import TreeSweeper
from .workloads import slab_wake


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--n", type=int, default=1 << 20)
    p.add_argument("--leaf", type=int, default=48)
    p.add_argument("--far-field", default="learned", choices=["m2p", "m2l", "learned"])
    p.add_argument("--repeat", type=int, default=0)
    a = p.parse_args(argv)
    pos, gam, sig, _ = slab_wake(a.n)
    d = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")  # noqa: E731
    P, G, S = d(pos), d(gam), d(sig)
    ts = TreeSweeper(theta=0.5, leaf_target=a.leaf)
    mlp = None
    if a.far_field == "learned":
        from .learned import FarFieldMLP
        mlp = FarFieldMLP.load()
    ts.set_far_field(a.far_field, mlp=mlp)
    ts.set_validation(0, 0.1)
    out = torch.empty((a.n, 3), dtype=torch.float64, device="cuda")
    ts.sweep(_capi.PAIR_VELOCITY, "winckelmans", P, G, S, a.n, out)
    ts.sweep(_capi.PAIR_STRETCH, "winckelmans", P, G, S, a.n, out, tgt_gamma=G)
    times = {"velocity": [], "stretch": []}
    for _ in range(a.repeat):
        for name, mode, tg in (("velocity", _capi.PAIR_VELOCITY, None),
                               ("stretch", _capi.PAIR_STRETCH, G)):
            ts.sweep(mode, "winckelmans", P, G, S, a.n, out, tgt_gamma=tg, check=True,
                     same_positions=True)
            local = ts.last_local_ms() if a.far_field != "m2p" else 0.0
            times[name].append((ts.last_eval_ms(), local))
    torch.cuda.synchronize()
    for name, t in times.items():
        if t:
            ev = sorted(x[0] for x in t)[len(t) // 2]
            lo = sorted(x[1] for x in t)[len(t) // 2]
            print(f"{name}: evaluation {ev:.3f} ms, local-expansion stage {lo:.3f} ms "
                  f"(median of {len(t)})")
    print("sweep case ok: max |S| =", float(out.abs().max()),
          "status", _capi.status_read_and_clear())


if __name__ == "__main__":
    main()
