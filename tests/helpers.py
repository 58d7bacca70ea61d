"""Shared helpers for the parity tests."""
import os

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


AFFINE_A = np.array([[0.8, 0.3, -0.2], [0.1, -0.5, 0.4], [-0.3, 0.2, 0.6]])


def affine_block(model):
    """A 16^3-particle block with the affine velocity field v = A (x - c) + b and no gravity.
    For particles 2.5 cells or more inside the block every node they read sees a full
    lattice, so GIMP reproduces the linear field: their first-step strain rate is sym(A)
    exactly.  Returns the scene and the mask of those particles."""
    from graphyt_gb300 import scenes
    sc = scenes.tiny_block(model=model, n_side=16, L=(2.5, 2.5, 2.5), gravity=(0.0, 0.0, 0.0))
    sc.materials[0]["viscosity"] = 2e5
    sc.materials[0]["yieldStress"] = 300.0
    sc.vel = (sc.pos - sc.pos.mean(axis=0)) @ AFFINE_A.T + np.array([0.05, -0.02, 0.01])
    lo, hi, d = sc.pos.min(axis=0), sc.pos.max(axis=0), 2.5 * sc.cellsize - 1e-9
    inner = np.all((sc.pos > lo + d) & (sc.pos < hi - d), axis=1)
    return sc, inner


def affine_block_stress(model, mat, dt):
    """Stress after one step from zero stress and zero strain under the strain rate sym(A):
    elastic, ConstitutiveModels.cpp:12-28 (1/3 written 0.3333); Newtonian, :41-62 (1/3 written
    0.33333, pressure K tr(strain), viscous terms multiplied by dt); perfect plasticity,
    :139-222 (1/3 written 0.33; von Mises trial stress, radial return of the increment
    dL = (q - Y) / 3G along the deviatoric flow direction)."""
    E = 0.5 * (AFFINE_A + AFFINE_A.T)
    er = np.array([E[0, 0], E[1, 1], E[2, 2], E[0, 1], E[1, 2], E[0, 2]])
    K, G, mu = mat["bulkMod"], mat["shearMod"], mat["viscosity"]
    out = np.empty(6)
    if model == 1:
        vol = 0.3333 * er[:3].sum()
        out[:3] = (2.0 * G * (er[:3] - vol) + 3.0 * K * vol) * dt
        out[3:] = 2.0 * G * er[3:] * dt
    elif model == 3:
        vol = 0.3300 * er[:3].sum()
        tr = np.empty(6)
        tr[:3] = (2.0 * G * (er[:3] - vol) + 3.0 * K * vol) * dt
        tr[3:] = 2.0 * G * er[3:] * dt
        q = np.sqrt(0.5 * ((tr[0] - tr[1]) ** 2 + (tr[1] - tr[2]) ** 2 + (tr[2] - tr[0]) ** 2)
                    + tr[3] ** 2 + tr[4] ** 2 + tr[5] ** 2)
        assert q > mat["yieldStress"]  # the case exercises the return
        dL = (q - mat["yieldStress"]) / (3.0 * G)
        pl = dL * (0.5 / q) * np.array([2 * tr[0] - tr[1] - tr[2], 2 * tr[1] - tr[2] - tr[0],
                                        2 * tr[2] - tr[0] - tr[1], 6 * tr[3], 6 * tr[4], 6 * tr[5]])
        ee = er - pl / dt
        out[:3] = (2.0 * G * (ee[:3] - vol) + 3.0 * K * vol) * dt
        out[3:] = 2.0 * G * ee[3:] * dt
    else:
        vol = 0.33333 * er[:3].sum()
        P = K * er[:3].sum() * dt
        out[:3] = P + mu * (2.0 - 2.0 / 3.0) * (er[:3] - vol) * dt
        out[3:] = 2.0 * mu * er[3:] * dt
    return out, er * dt


def perturbed(scene, eps, seed):
    """A copy of the scene whose initial positions are scaled by (1 + eps * N(0, 1)), seeded."""
    import copy
    sp = copy.deepcopy(scene)
    rng = np.random.default_rng(seed)
    sp.pos = scene.pos * (1.0 + eps * rng.standard_normal(scene.pos.shape))
    return sp


def _ensemble_member(args):
    """One FP64 run (in a worker process): the fields by particle id at each horizon."""
    scene, horizons, fields, threads = args
    import os
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle.oracle import Oracle
    o = Oracle(scene, "port", mode=1)
    out = {}
    for k in range(1, max(horizons) + 1):
        o.step()
        if k in horizons:
            out[k] = {f: o.pfield(f) for f in fields}
    return out


def oracle_ensemble(scene, horizons, fields, members=8, eps=1e-7):
    """The FP64 restatement run from the scene and from `members` copies with initial positions
    perturbed by a relative eps (seeds 100, 101, ...), the runs spread over the host's cores in
    spawned worker processes.  Returns {horizon: (base fields, spread)} where spread[f] is the
    largest relative L2 distance between two of the runs (perturbed or not): how far apart
    rounding-sized input changes carry the reference itself by that step."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    horizons = sorted(set(int(h) for h in horizons))
    scenes_ = [scene] + [perturbed(scene, eps, 100 + s) for s in range(members)]
    cores = os.cpu_count() or 1
    threads = max(1, cores // len(scenes_))
    with ProcessPoolExecutor(max_workers=min(len(scenes_), cores), mp_context=mp.get_context("spawn")) as ex:
        runs = list(ex.map(_ensemble_member, [(s, horizons, fields, threads) for s in scenes_]))
    out = {}
    for h in horizons:
        base = runs[0][h]
        spread = {}
        for f in fields:
            mem = [r[h][f] for r in runs[1:]]
            pair = max(rel_l2(a, b) for i, a in enumerate(mem) for b in mem[i + 1:])
            spread[f] = max(pair, max(rel_l2(m, base[f]) for m in mem))
        out[h] = (base, spread)
    return out
