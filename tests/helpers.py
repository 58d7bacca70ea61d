"""Shared helpers for the parity tests."""
import numpy as np


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return num / den if den > 0 else num


def run_gpu(scene, nsteps, options=None):
    from graphyt_gb300 import graphyt
    s = graphyt.from_scene(scene, options=options)
    dt = s.dt
    for k in range(nsteps):
        s.iterate_GPU(k * dt, k)
    s.Synchronise()
    return s


def run_oracle(scene, nsteps, kind="port"):
    from oracle.oracle import Oracle
    o = Oracle(scene, kind, mode=1)
    o.run(nsteps)
    return o
