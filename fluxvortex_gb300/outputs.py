"""Output files in the layouts the reference's own scripts write and read.

- Force histories: ``t_<tag>``, ``cl_<tag>``, ``cdi_<tag>`` float64 arrays per
  run, the layout of figures/flapping_results.npz
  (tests/benchmark_flapping.py:251-257, read by tests/plot_flapping.py);
  ``save_force_history`` merges new runs into an existing file.
- ``force_coefficients_W``: PteraSoftware's wind-axes coefficient vector as
  the reference reads it (tests/benchmark_flapping.py:162-163: CL = -c[2],
  CDi = -c[0]), i.e. c = [-CDi, CY, -CL].
- Particle snapshots: pos, alpha, sigma, age of the live particles and the
  time, one ``.npz`` per snapshot.
- Flutter sweeps: the tip heave / twist histories of every airspeed with the
  airspeeds, time step, growth rates and flutter speed (``save_flutter_tips``);
  and the layout of the reference's figures/flutter_data.npz
  (tests/animate_flutter.py:161-168, ``save_flutter_data``): every beam node's
  heave and twist per recorded step at a stable and a fluttering airspeed,
  ``w_stable``, ``theta_stable``, ``w_flutter``, ``theta_flutter`` (steps x
  nodes), the nodes' span stations ``y_nodes`` and the time step ``dt``.
"""
from __future__ import annotations

import os

import numpy as np


def force_coefficients_W(cl, cdi, cy=None):
    """c = [-CDi, CY, -CL] (CY = 0 when not given), broadcast over histories."""
    cl = np.asarray(cl, dtype=np.float64)
    cdi = np.asarray(cdi, dtype=np.float64)
    cy = np.zeros_like(cl) if cy is None else np.asarray(cy, dtype=np.float64)
    return np.stack([-cdi, cy, -cl], axis=-1)


def _history(run, dt=None):
    """(t, cl, cdi) of a HybridStep-like object (``cl``, ``cdi``, ``cfg.dt``)
    or of a (t, cl, cdi) tuple."""
    if isinstance(run, (tuple, list)):
        t, cl, cdi = (np.asarray(x, dtype=np.float64) for x in run)
        return t, cl, cdi
    cl = np.asarray(run.cl, dtype=np.float64)
    cdi = np.asarray(run.cdi, dtype=np.float64)
    step = dt if dt is not None else run.cfg.dt
    return np.arange(cl.size) * step, cl, cdi


def save_force_history(path, runs, dt=None):
    """Writes (or adds to) ``path``: for each tag of ``runs`` (tag -> run),
    t_<tag>, cl_<tag>, cdi_<tag>.  Keys already in the file and not among the
    new tags are kept."""
    out = {}
    if os.path.exists(path):
        with np.load(path, allow_pickle=False) as old:
            out.update({k: old[k] for k in old.files})
    for tag, run in runs.items():
        t, cl, cdi = _history(run, dt)
        out[f"t_{tag}"], out[f"cl_{tag}"], out[f"cdi_{tag}"] = t, cl, cdi
    np.savez(path, **out)


def load_force_history(path):
    """tag -> (t, cl, cdi) for every complete triple in the file."""
    with np.load(path, allow_pickle=False) as z:
        tags = sorted(k[2:] for k in z.files if k.startswith("t_"))
        return {tag: (z[f"t_{tag}"], z[f"cl_{tag}"], z[f"cdi_{tag}"]) for tag in tags
                if f"cl_{tag}" in z.files and f"cdi_{tag}" in z.files}


def save_particles(path, field, t=None):
    """The live particles of a VortexParticleField (host copies)."""
    np.savez(path, pos=field.positions, alpha=field.gammas, sigma=field.sigmas, age=field.ages,
             np=np.int64(field.np), t=np.float64(np.nan if t is None else t))


def save_flutter_tips(path, sweep):
    """Tip histories of a FlutterSweep: w_tip_<V>, theta_tip_<V> per airspeed
    (V formatted with one decimal), velocities, dt, sigma, flutter_speed."""
    w, th = sweep.histories()
    out = {"velocities": np.asarray(sweep.V, dtype=np.float64),
           "dt": np.float64(sweep.cfg.dt),
           "sigma": np.asarray(sweep.sigma(), dtype=np.float64),
           "flutter_speed": np.float64(sweep.flutter_speed())}
    for V, a, b in zip(sweep.V, w, th):
        out[f"w_tip_{V:.1f}"] = np.asarray(a, dtype=np.float64)
        out[f"theta_tip_{V:.1f}"] = np.asarray(b, dtype=np.float64)
    np.savez(path, **out)


def save_flutter_data(path, sweep, v_stable, v_flutter):
    """The reference's flutter_data.npz layout from a FlutterSweep made with
    node_histories=True: the environments whose airspeeds are nearest
    ``v_stable`` and ``v_flutter``."""
    V = np.asarray(sweep.V, dtype=np.float64)
    es = int(np.argmin(np.abs(V - v_stable)))
    ef = int(np.argmin(np.abs(V - v_flutter)))
    ws, ts = sweep.node_histories(es)
    wf, tf = sweep.node_histories(ef)
    np.savez_compressed(path, w_stable=ws, theta_stable=ts, w_flutter=wf, theta_flutter=tf,
                        y_nodes=np.asarray(sweep.beam.y_nodes, dtype=np.float64),
                        dt=np.float64(sweep.cfg.dt))


def load_flutter_data(path):
    """The two histories of a flutter_data.npz as the reference's animation
    reads them: {"stable"|"flutter": {w_history, theta_history, y_nodes, dt}}."""
    with np.load(path, allow_pickle=False) as z:
        y, dt = z["y_nodes"], float(z["dt"])
        return {tag: {"w_history": z[f"w_{tag}"], "theta_history": z[f"theta_{tag}"],
                      "y_nodes": y, "dt": dt} for tag in ("stable", "flutter")}
