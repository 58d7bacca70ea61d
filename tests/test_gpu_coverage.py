"""GPU parity on paths the main parity file does not reach: the periodic node fold, the
turbulent-liquid model, contact normals, the particle BC family, and multi-body problems
between sorts.  Same tolerances as test_gpu_parity.py (FP32 GPU against the FP64 oracle)."""
import numpy as np
import pytest

from graphyt_gb300 import scenes
from tests.helpers import rel_l2, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

ONE_STEP_TOL = 1e-5
MANY_STEP_TOL = 1e-3


def _compare(gpu, ref, fields, tol):
    for f in fields:
        a, b = gpu._get_particles(f), ref.pfield(f)
        if np.linalg.norm(b) == 0:
            assert np.max(np.abs(a)) < 1e-9, f
        else:
            assert rel_l2(a, b) <= tol, (f, rel_l2(a, b))


def test_periodic_fold_seam(gpu_lib, oracle_built):
    """A block whose stencils reach the last three node layers on every axis: their sums are
    folded onto the first three (Grid.cpp:310-795) and read back by G2P.  The block stays
    below the wrap threshold L - 2 cellsize, so no particle wraps (a wrapped particle is
    invisible to the reference's P2G until its next sort)."""
    sc = scenes.tiny_block(model=1, n_side=6)
    sc.pos += np.array([0.35, 0.40, 0.40])
    assert sc.pos.max() < sc.L[0] - 2 * sc.cellsize - 0.02
    for steps, tol in ((2, ONE_STEP_TOL), (20, MANY_STEP_TOL)):
        _compare(run_gpu(sc, steps), run_oracle(sc, steps), ("vel", "stress", "pos"), tol)


def test_turbulent_liquid(gpu_lib, oracle_built):
    """Material model 5, turbulentLiquid (ConstitutiveModels.cpp:66-126)."""
    sc = scenes.tiny_block(model=5)
    for steps, tol in ((2, ONE_STEP_TOL), (30, MANY_STEP_TOL)):
        _compare(run_gpu(sc, steps), run_oracle(sc, steps), ("vel", "stress", "density"), tol)


def test_contact_normals(gpu_lib, oracle_built):
    """Two bodies in contact with per-particle contact normals kept (getNormalsArr,
    Extrapolation.cpp:311-355)."""
    sc = scenes.two_blocks()
    gpu = run_gpu(sc, 12, options=dict(track_normals=1))
    ref = run_oracle(sc, 12)
    _compare(gpu, ref, ("vel", "stress"), MANY_STEP_TOL)
    a, b = gpu._get_particles("normals"), ref.pfield("normals")
    assert np.linalg.norm(b) > 0
    assert rel_l2(a, b) <= MANY_STEP_TOL


def test_particle_bc_family(gpu_lib, oracle_built):
    """Velocity, force, sine-ramped and stress particle BCs (TimeIntegration.cpp:177-296) on
    disjoint slices of one block."""
    sc = scenes.tiny_block(model=1, n_side=8, gravity=(0.0, 0.0, -9.81))
    x = sc.pos[:, 0]
    edges = np.quantile(x, np.linspace(0, 1, 9))
    kinds = [("mp_vx", (0.2, 0, 0, 0)), ("mp_vy", (-0.1, 0, 0, 0)), ("mp_fx", (3e-3, 0, 0, 0)),
             ("mp_fz", (-2e-3, 0, 0, 0)), ("mp_vxsin", (0.1, 5.0, 0, 0)), ("mp_vx_vy", (0.05, -0.05, 0, 0)),
             ("mp_fx_fy", (1e-3, 2e-3, 0, 0)), ("none", (0, 0, 0, 0))]
    for k, (name, val) in enumerate(kinds):
        sel = (x >= edges[k]) & (x <= edges[k + 1]) if k == len(kinds) - 1 else (x >= edges[k]) & (x < edges[k + 1])
        sc.pbc_type[sel] = scenes.BC[name]
        sc.pbc_val[sel] = val
    for steps, tol in ((2, ONE_STEP_TOL), (15, MANY_STEP_TOL)):
        _compare(run_gpu(sc, steps), run_oracle(sc, steps), ("vel", "stress", "pos"), tol)


def test_multibody_between_sorts(gpu_lib):
    """Multi-body contact with the particles re-ordered only every fourth step agrees with
    sorting every step (the order is a performance choice)."""
    sc = scenes.two_blocks()
    a = run_gpu(sc, 14, options=dict(sort_every=1))
    b = run_gpu(sc, 14, options=dict(sort_every=4))
    for f in ("vel", "stress"):
        assert rel_l2(a._get_particles(f), b._get_particles(f)) < 1e-5, f


def test_nonfinite_state_is_reported(gpu_lib):
    """A particle whose velocity is not finite makes the step report GY_ERR_NONFINITE at the
    next synchronisation (check_finite); the kernels' own clamps keep every index in range."""
    from graphyt_gb300 import _lib, graphyt
    sc = scenes.tiny_block(model=1)
    sc.vel[0] = np.nan
    with pytest.raises(_lib.GraphytGPUError) as e:
        s = graphyt.from_scene(sc, options=dict(check_finite=1))
        for k in range(3):
            s.iterate_GPU(k * s.dt, k)
        s.Synchronise()
    assert e.value.code in (_lib.GY_ERR_NONFINITE, _lib.GY_ERR_ARG)


def test_full_size_dam_break_mirror_symmetry(gpu_lib):
    """Size-independent property at the benchmark's full size (11,995,200 particles): the dam
    break is mirror-symmetric about the domain's mid-plane in y, so after ten steps every
    particle's velocity mirrors its partner's to FP32 summation noise."""
    sc = scenes.dam_break(scale=1.0)
    s = run_gpu(sc, 10)
    v = s._get_particles("vel")
    p0 = sc.pos
    psep = sc.psep
    ix = np.floor(p0 / psep).astype(np.int64)  # lattice points sit at (k + 1/2) psep
    iy_m = ix[:, 1].min() + ix[:, 1].max() - ix[:, 1]
    ny = ix[:, 1].max() + 2
    nz = ix[:, 2].max() + 2
    key = (ix[:, 0] * ny + ix[:, 1]) * nz + ix[:, 2]
    mkey = (ix[:, 0] * ny + iy_m) * nz + ix[:, 2]
    order = np.argsort(key)
    pos_in_sorted = np.searchsorted(key[order], mkey)
    mate = order[pos_in_sorted]
    assert np.array_equal(key[mate], mkey)
    assert np.linalg.norm(v) > 0
    # v_x, v_z equal and v_y opposite on mirror pairs
    scale = np.linalg.norm(v)
    assert np.linalg.norm(v[:, 0] - v[mate, 0]) <= 1e-4 * scale
    assert np.linalg.norm(v[:, 2] - v[mate, 2]) <= 1e-4 * scale
    assert np.linalg.norm(v[:, 1] + v[mate, 1]) <= 1e-4 * scale
    st = s.stats()
    m = s._get_particles("mass").sum()
    assert abs(st["mass"] - m) <= 1e-9 * m


def _fp64_stats(s):
    m = s._get_particles("mass")
    v = s._get_particles("vel").reshape(-1, 3)
    sig = s._get_particles("stress").reshape(-1, 6)
    eps = s._get_particles("strain").reshape(-1, 6)
    rho = s._get_particles("density")
    se = (sig[:, :3] * eps[:, :3]).sum(1) + 2.0 * (sig[:, 3:] * eps[:, 3:]).sum(1)
    return dict(mass=m.sum(), momentum=(m[:, None] * v).sum(0), kinetic=0.5 * (m * (v * v).sum(1)).sum(),
                strain_energy=0.5 * (m / rho * se).sum(), pscale=(m * np.abs(v).sum(1)).sum(),
                sscale=0.5 * (m / rho * np.abs(se)).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("scene", ["dam_break", "two_blocks", "brazilian_disc"])
def test_step_fused_stats_match_separate_sum(gpu_lib, tmp_path, scene):
    """The conservation sums a step's G2P accumulates equal a separate pass over the state it
    wrote (the pass a state load forces) and FP64 sums of the fetched fields."""
    sc = {"dam_break": lambda: scenes.dam_break(scale=0.125),
          "two_blocks": lambda: scenes.two_blocks(),
          "brazilian_disc": lambda: scenes.brazilian_disc(scale=0.25)}[scene]()
    s = run_gpu(sc, 7)
    fused = s.stats()
    path = str(tmp_path / "state.bin")
    s.save(path)
    s.load(path)
    full = s.stats()
    ref = _fp64_stats(s)
    for st in (fused, full):
        assert abs(st["mass"] - ref["mass"]) <= 1e-12 * ref["mass"]
        assert np.max(np.abs(np.array(st["momentum"]) - ref["momentum"])) <= 1e-5 * ref["pscale"]
        assert abs(st["kinetic"] - ref["kinetic"]) <= 1e-5 * ref["kinetic"] + 1e-30
        assert abs(st["strain_energy"] - ref["strain_energy"]) <= 1e-5 * ref["sscale"] + 1e-30
        assert st["steps"] == 7
    assert ref["kinetic"] > 0


def _single_particle_scene(offset):
    h = 0.1
    pos = np.array([[0.5 + offset[0] * h, 0.5 + offset[1] * h, 0.5 + offset[2] * h]])
    sc = scenes.Scene("one", [1.0, 1.0, 1.0], h, h / 2, pos, np.zeros(1, np.int32), np.zeros(1, np.int32),
                      [scenes.material(model=1)], gravity=[0.0, 0.0, -9.81])
    sc.vel = np.array([[0.3, -0.2, 0.1]])
    return scenes._finish(sc, None)


@pytest.mark.gpu
@pytest.mark.parametrize("offset", [(0.25, 0.25, 0.25), (0.6, 0.1, 0.9), (0.999, 0.001, 0.5)])
def test_single_particle(gpu_lib, oracle_built, offset):
    """One particle, anywhere in its cell (its own run, segment and node tile) falls and
    drifts as in the restatement."""
    sc = _single_particle_scene(offset)
    gpu = run_gpu(sc, 20)
    ref = run_oracle(sc, 20)
    for f in ("vel", "pos"):
        assert rel_l2(gpu._get_particles(f), ref.pfield(f)) <= 1e-5, f
    # a lone particle translates rigidly: its strain rate is the gradient sum of one velocity,
    # zero up to rounding (FP64 ~1e-17, FP32 ~1e-8), so the stress stays at rounding level
    assert np.max(np.abs(gpu._get_particles("stress"))) < 1.0
    assert np.max(np.abs(ref.pfield("stress"))) < 1.0


@pytest.mark.gpu
def test_no_particles(gpu_lib):
    """A solver without particles initialises, steps and reports zero sums."""
    sc = scenes.Scene("empty", [1.0, 1.0, 1.0], 0.1, 0.05, np.zeros((0, 3)), np.zeros(0, np.int32),
                      np.zeros(0, np.int32), [scenes.material(model=1)])
    sc = scenes._finish(sc, None)
    s = run_gpu(sc, 5)
    st = s.stats()
    assert st["mass"] == 0.0 and st["kinetic"] == 0.0 and st["steps"] == 5
    assert s._get_particles("vel").shape[0] == 0


def test_weibull_flaws_match_oracle(gpu_lib, oracle_built):
    """Per-particle Weibull activation strains (scene weibull_flaws, seed 0) on the damage
    block: the GPU's damage gate uses the particle's own scale -- the state after two steps
    within 1e-5 of the FP64 restatement with the same scales, after 20 steps within the FP64
    ensemble's reach (the damage gate makes this scene ill-conditioned past a few steps)."""
    from tests.helpers import oracle_ensemble
    sc = scenes.damage_block(n_side=12, weibull_seed=0)
    assert np.any(sc.flaw != 1.0)
    gpu = run_gpu(sc, 2)
    ref = run_oracle(sc, 2)
    for f in ("vel", "stress", "damage"):
        assert rel_l2(gpu._get_particles(f), ref.pfield(f)) <= 1e-5, f
    ens = oracle_ensemble(sc, (20,), ("vel", "stress", "damage"), eps=1e-6)
    base, spread = ens[20]
    gpu = run_gpu(sc, 20)
    for f in ("vel", "stress", "damage"):
        assert rel_l2(gpu._get_particles(f), base[f]) <= max(1e-3, 2.0 * spread[f]), f


def test_flaw_scale_one_equals_plain_run(gpu_lib):
    """A flaw table of ones is the reference's deterministic e_min: the run equals the run
    without a table to FP32 summation order."""
    sc = scenes.damage_block(n_side=12)
    plain = run_gpu(sc, 20)
    sc.flaw = np.ones(sc.n)
    sc.flaw[0] = 1.0 + 2.0 ** -40  # a table is built (one scale differs from 1 below FP32 resolution)
    ones = run_gpu(sc, 20)
    for f in ("vel", "stress", "damage"):
        assert rel_l2(ones._get_particles(f), plain._get_particles(f)) <= 2e-6, f
