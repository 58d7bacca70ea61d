"""Generate the golden fixtures in this folder from the reference itself.

Runs the unmodified reference sources (oracle/_ref/libgyref.so, built by oracle/Makefile
from the reference tree) on the seeded scenes of graphyt_gb300.scenes and stores the final
particle state by particle id.  The fixtures let tests pin the oracle and the GPU path on
machines where the reference tree is absent.

    python tests/golden/make_golden.py [case ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from graphyt_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402

FIELDS = ["pos", "vel", "stress", "density", "strain", "eqps", "pstrain", "damage", "disp"]
THERMAL_FIELDS = ["temp", "tempgrad"]

# name -> (scene factory, steps, max stored particles)
CASES = {
    "tiny_elastic": (lambda: scenes.tiny_block(model=1), 40, None),
    "tiny_newtonian": (lambda: scenes.tiny_block(model=2), 40, None),
    "tiny_vonmises": (lambda: scenes.tiny_block(model=3), 40, None),
    "tiny_druckerprager": (lambda: scenes.tiny_block(model=4), 40, None),
    "cube_particle_bc": (lambda: scenes.elastic_cube("particle"), 60, 2000),
    "cube_nodal_literal": (lambda: scenes.elastic_cube("nodal"), 30, 500),
    "cube_nodal_fixed": (lambda: scenes.elastic_cube("fixed"), 30, 2000),
    "dam_break_coarse": (lambda: scenes.dam_break(scale=0.125), 30, 2000),
    "brazilian_coarse": (lambda: scenes.brazilian_disc(scale=0.1), 20, 3000),
    "damage_block": (lambda: scenes.damage_block(), 40, None),
    "two_blocks": (lambda: scenes.two_blocks(), 40, None),
    "two_blocks_rigid": (lambda: scenes.two_blocks(rigid_second=True), 40, None),
    "block_2d_elastic": (lambda: scenes.block_2d(model=1), 200, None),
    "block_2d_dp": (lambda: scenes.block_2d(model=4), 200, None),
    "block_2d_newtonian": (lambda: scenes.block_2d(model=2), 200, None),
    "block_2d_vonmises": (lambda: scenes.block_2d(model=3), 200, None),
    "block_2d_turbulent": (lambda: scenes.block_2d(model=5), 200, None),
    "thermal_block": (lambda: scenes.thermal_block(), 30, None),
    "thermal_2d": (lambda: scenes.thermal_2d(), 40, None),
    "disk_impact_2d": (lambda: scenes.disk_impact_2d(), 300, None),
}


def fields_for(name):
    return FIELDS + (THERMAL_FIELDS if name.startswith("thermal") else [])


def generate(name, kind="ref"):
    make, steps, cap = CASES[name]
    sc = make()
    o = oracle.Oracle(sc, kind, mode=1)
    o.run(steps)
    ids = np.arange(sc.n)
    if cap is not None and sc.n > cap:
        ids = np.linspace(0, sc.n - 1, cap).astype(np.int64)
    out = {"ids": ids, "steps": np.int64(steps), "dt": np.float64(o.dt), "n": np.int64(sc.n)}
    for f in fields_for(name):
        out[f] = o.pfield(f)[ids]
    return out


def main(names=None):
    if not oracle.available("ref"):
        oracle.build()
    for name in names or CASES:
        data = generate(name, "ref")
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, int(data["n"]), "particles,", int(data["steps"]), "steps")


if __name__ == "__main__":
    main(sys.argv[1:])
