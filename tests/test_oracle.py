"""CPU tests: the oracle against the reference and its golden vectors, plus known answers.

The oracle (oracle/gy_oracle.c) is pinned two ways: against the reference library
compiled from the reference sources (where the reference tree exists), and against the
golden fixtures in tests/golden that the reference produced (everywhere).
"""
import glob
import os

import numpy as np
import pytest

from graphyt_gb300 import scenes
from oracle import oracle
from tests.golden import make_golden
from tests.helpers import affine_block, affine_block_stress, rel_l2

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_port_matches_reference_goldens(oracle_built, name):
    """The FP64 restatement reproduces the reference's golden outputs to rounding."""
    path = os.path.join(GOLDEN, name + ".npz")
    gold = np.load(path)
    got = make_golden.generate(name, kind="port")
    for f in make_golden.fields_for(name):
        a, b = got[f], gold[f]
        if np.linalg.norm(b) == 0:
            assert np.array_equal(a, b), f
        else:
            assert rel_l2(a, b) <= 1e-12, (name, f, rel_l2(a, b))


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libgyref.so"))
                    and not os.path.isdir(oracle.REFERENCE_DIR), reason="reference tree not available")
def test_harness_mode_matches_literal_iterate_cpu(oracle_built):
    """The harness sequence (stable (cell, id) sort) equals Solver::iterate_CPU up to the
    summation order std::sort leaves inside a cell."""
    from oracle.oracle import Oracle, available
    if not available("ref"):
        pytest.skip("reference library not built")
    sc = scenes.elastic_cube("particle")
    lit = Oracle(sc, "ref", mode=0)
    har = Oracle(sc, "ref", mode=1)
    lit.run(25)
    har.run(25)
    for f in ["vel", "stress", "pos", "density"]:
        assert rel_l2(har.pfield(f), lit.pfield(f)) < 1e-12


def test_golden_files_present():
    names = {os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))}
    assert set(make_golden.CASES) <= names


# ---------------------------------------------------------------------------------------
# known-answer tests from the reference's mathematics

def test_gimp_partition_of_unity(oracle_built):
    """Sum of GIMP shape values is 1 and of gradients 0 for interior particles
    (Extrapolation.cpp:572-644)."""
    from oracle.oracle import gimp_grad, gimp_shape
    h, lp = 0.05, 0.0125
    rng = np.random.default_rng(3)
    for xp in rng.uniform(0.3, 0.7, 200):
        nodes = np.arange(0, 21) * h
        S = sum(gimp_shape(xn - xp, h, lp) for xn in nodes)
        G = sum(gimp_grad(xn - xp, h, lp, xp) for xn in nodes)
        assert abs(S - 1.0) < 1e-12
        assert abs(G) < 1e-9


def test_gimp_gradient_is_shape_derivative(oracle_built):
    from oracle.oracle import gimp_grad, gimp_shape
    h, lp = 0.1, 0.025
    for d in np.linspace(-0.124, 0.124, 97):
        xp = 0.5
        # gradient with respect to the particle coordinate = -dS/d(dist)
        eps = 1e-7
        num = -(gimp_shape(d + eps, h, lp) - gimp_shape(d - eps, h, lp)) / (2 * eps)
        assert abs(gimp_grad(d, h, lp, xp) - num) < 1e-4


def test_sym_eigen_reconstructs(oracle_built):
    from oracle.oracle import sym_eigen
    rng = np.random.default_rng(7)
    for _ in range(50):
        a = rng.standard_normal((3, 3)) * 1e7
        a = a + a.T
        d, V = sym_eigen(a)
        assert np.all(np.diff(d) >= 0)
        assert np.allclose(V @ np.diag(d) @ V.T, a, rtol=0, atol=1e-6 * np.abs(a).max())
        assert np.allclose(d, np.linalg.eigvalsh(a), rtol=1e-12, atol=1e-6)


def test_drucker_prager_return_lands_on_yield_surface(oracle_built):
    """After a plastic DP step the returned stress satisfies F = sqrt(J2) + eta p - xi c(eps_p) = 0
    (ConstitutiveModels.cpp:321-344, 398-403) for the non-softened, non-apex branch."""
    import math
    phi, psi = 30.0, 10.0
    p_ = phi * 3.14159 / 180
    eta = 6 * math.sin(p_) / (math.sqrt(3) * (3 - math.sin(p_)))
    xi = 6 * math.cos(p_) / (math.sqrt(3) * (3 - math.sin(p_)))
    sc = scenes.tiny_block(model=4, n_side=6, gravity=(0, 0, -200.0), vel=(0, 0, 0))
    sc.materials = [scenes.material(bulkMod=1e6, shearMod=4e5, density=1200.0, cohesion=500.0, phi=phi,
                                    psi=psi, criticalStrain=1e9, model=4)]
    from oracle.oracle import Oracle
    o = Oracle(sc, "port")
    o.run(40)
    s = o.pfield("stress")
    eq = o.pfield("eqps")
    plastic = eq > 0
    assert plastic.any()
    p = s[plastic, :3].mean(axis=1)
    dev = s[plastic].copy()
    dev[:, :3] -= p[:, None]
    J2 = 0.5 * (dev[:, 0] ** 2 + dev[:, 1] ** 2 + dev[:, 2] ** 2) + dev[:, 3] ** 2 + dev[:, 4] ** 2 + dev[:, 5] ** 2
    c = 500.0 - eq[plastic] * (500.0 / 1e9)
    F = np.sqrt(J2) + eta * p - xi * c
    # particles that yielded in the last step sit on the surface; others are inside
    assert np.all(F <= 1e-6 * 500.0 + 1e-9)
    assert np.min(np.abs(F)) < 1e-6 * 500.0


def test_grady_kipp_growth_law():
    """D^(1/3) grows by dt ((m+3)/3) alpha^(1/3) eps^(m/3) (DamageModels.cpp:101-109)."""
    import math
    m, k, Cg, dt, D0, eps = 9.0, 5e32, 1867.4, 4e-8, 0.2, 2e-3
    alpha = 8 * 3.14159 * Cg ** 3 * k / ((m + 1) * (m + 2) * (m + 3))
    rate = ((m + 3) / 3) * alpha ** (1 / 3) * eps ** (m / 3)
    D1 = (D0 ** (1 / 3) + dt * rate) ** 3
    assert D1 > D0
    assert math.isclose((D1 ** (1 / 3) - D0 ** (1 / 3)) / dt, rate, rel_tol=1e-9)


def test_periodic_fold_pairs(oracle_built):
    """After a step, node i and node N-3+i carry the same mass on every axis (Grid.cpp:317-329)."""
    from oracle.oracle import Oracle
    sc = scenes.tiny_block(model=1, n_side=6)
    # move the block onto the periodic seam in x
    sc.pos[:, 0] += 0.85
    o = Oracle(sc, "port")
    o.step()
    nx, ny, nz = sc.dims()
    m = o.nfield("mass").reshape(nz, ny, nx)
    for i in range(3):
        assert np.array_equal(m[:, :, i], m[:, :, nx - 3 + i])
        assert np.array_equal(m[:, i, :], m[:, ny - 3 + i, :])
        assert np.array_equal(m[i, :, :], m[nz - 3 + i, :, :])


def test_do_nothing_invariant_3d(oracle_built):
    """3D restatement of test/test_2d_do_nothing.py:92-99: a block at rest with no BC and no
    gravity keeps zero displacement and zero stress exactly."""
    from oracle.oracle import Oracle
    sc = scenes.tiny_block(model=1, n_side=6, gravity=(0, 0, 0), vel=(0, 0, 0))
    sc.vel[:] = 0.0
    o = Oracle(sc, "port")
    o.run(50)
    assert np.all(o.pfield("disp") == 0.0)
    assert np.all(o.pfield("stress") == 0.0)


def test_literal_nodal_z_bcs_leave_cube_at_rest(oracle_built):
    """grid_vz dispatches to an empty body (Grid.cpp:872-873, 1032-1034): the nodal-BC cube
    does not move."""
    gold = np.load(os.path.join(GOLDEN, "cube_nodal_literal.npz"))
    assert np.all(gold["vel"] == 0.0) and np.all(gold["stress"] == 0.0)


def test_scene_counts():
    """Particle counts of the named workloads."""
    assert scenes.elastic_cube("particle").n == 8000
    pts = scenes.lattice_box([0.02, 0.02, 0.02], [1.02, 1.98, 0.785], 0.005)
    assert len(pts) == 200 * 392 * 153


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libgyref.so"))
                    and not os.path.isdir(oracle.REFERENCE_DIR), reason="reference tree not available")
def test_thermal_harness_matches_literal_between_sorts(oracle_built):
    """Heat conduction: the harness sequence and the restatement equal Solver::iterate_CPU
    while no sort has moved a temperature gradient (steps 1-9: the step-1 sort sees the
    all-zero initial gradients).  A run through step 1's sort of step 0's gradients differs,
    since the reference's sort copies one gradient component per slot
    (Extrapolation.cpp:446, 485)."""
    from oracle.oracle import Oracle, available
    if not available("ref"):
        pytest.skip("reference library not built")
    sc = scenes.thermal_block()

    def temp_after(kind, mode, steps):
        o = Oracle(sc, kind, mode=mode)
        for k in steps:
            o.step(step=k)
        return o.pfield("temp")

    clean = range(1, 10)
    lit, har, port = temp_after("ref", 0, clean), temp_after("ref", 1, clean), temp_after("port", 1, clean)
    dT = np.linalg.norm(har - sc.temp)
    assert dT > 1.0
    assert np.linalg.norm(lit - har) <= 1e-12 * dT
    assert np.linalg.norm(port - har) <= 1e-12 * dT
    garbled = range(0, 9)
    assert np.linalg.norm(temp_after("ref", 0, garbled) - temp_after("ref", 1, garbled)) > 1e-3 * dT


@pytest.mark.parametrize("model", [1, 2, 3])
def test_constitutive_first_step_known_answer(oracle_built, model):
    """Under an affine velocity field the first step's strain rate is sym(A) at interior
    particles, so their stress and strain follow the closed forms of the elastic, Newtonian
    and perfectly plastic laws with the reference's literal constants (0.3333, 0.33333, 0.33
    for 1/3)."""
    from oracle.oracle import Oracle
    sc, inner = affine_block(model)
    o = Oracle(sc, "port")
    o.run(1)
    want_s, want_e = affine_block_stress(model, sc.materials[0], o.dt)
    s, e = o.pfield("stress")[inner], o.pfield("strain")[inner]
    assert inner.sum() == 216
    assert np.abs(s - want_s).max() <= 1e-12 * np.abs(want_s).max()
    assert np.abs(e - want_e).max() <= 1e-12 * np.abs(want_e).max()


def test_flaw_scale_one_is_the_reference(oracle_built):
    """A flaw table of ones (every particle's activation strain the deterministic
    (V k)^(-1/m), DamageModels.cpp:102-103) reproduces the reference's golden damage block."""
    import ctypes as C
    from oracle.oracle import Oracle
    gold = np.load(os.path.join(GOLDEN, "damage_block.npz"))
    make, steps, _ = make_golden.CASES["damage_block"]
    sc = make()
    o = Oracle(sc, "port", mode=1)
    ids = np.arange(sc.n, dtype=np.int32)
    ones = np.ones(sc.n)
    o.lib.gyo_set_particle_flaws(o.h, sc.n, ids.ctypes.data_as(C.POINTER(C.c_int)),
                                 ones.ctypes.data_as(C.POINTER(C.c_double)))
    o.run(int(gold["steps"]))
    for f in ("stress", "damage", "vel", "eqps"):
        assert rel_l2(o.pfield(f)[gold["ids"]], gold[f]) <= 1e-12, f


def test_weibull_flaw_draw():
    """weibull_flaws: w = (-ln U)^(1/m) for the Grady-Kipp material, 1 elsewhere; w^m is then
    exponentially distributed with mean 1 (the reference's e_min is its w = 1 case)."""
    sc = scenes.brazilian_disc(scale=0.1, weibull_seed=0)
    m = sc.materials[0]["damageM"]
    rock = sc.mat == 0
    assert np.all(sc.flaw[~rock] == 1.0)
    x = sc.flaw[rock] ** m
    assert abs(x.mean() - 1.0) < 0.05 and abs(np.median(x) - np.log(2.0)) < 0.05
    again = scenes.brazilian_disc(scale=0.1, weibull_seed=0)
    assert np.array_equal(sc.flaw, again.flaw)


def test_weibull_flaws_change_damage(oracle_built):
    """With Weibull scales (m = 9: w spread over about 0.8-1.15) the damage field departs from
    the deterministic threshold's, and the particles whose damage has grown are those with
    the smaller scales."""
    from tests.helpers import run_oracle
    plain = run_oracle(scenes.damage_block(n_side=8), 10)
    wb_scene = scenes.damage_block(n_side=8, weibull_seed=0)
    wb = run_oracle(wb_scene, 10)
    d0, d1 = plain.pfield("damage"), wb.pfield("damage")
    assert rel_l2(d1, d0) > 1e-3
    assert (d1 > 0).sum() != (d0 > 0).sum()
    grown = d1 > 0
    assert grown.any() and (~grown).any()
    assert np.median(wb_scene.flaw[grown]) < np.median(wb_scene.flaw[~grown])
