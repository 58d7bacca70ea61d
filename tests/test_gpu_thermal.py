"""GPU parity of the heat conduction terms (P2G Extrapolation.cpp:280-283, G2P :358-362,
update TimeIntegration.cpp:49-50) against the oracle and the reference's golden fixture."""
import os

import numpy as np
import pytest

from graphyt_gb300 import scenes
from tests.golden import make_golden
from tests.helpers import rel_l2, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# FP32 temperature: the change of T over a run is compared relative to its own size
STEP_TOL = 1e-4
MANY_STEP_TOL = 1e-3


def _dT(temp, scene):
    return temp - scene.temp


def test_thermal_one_step_parity(gpu_lib, oracle_built):
    """After two steps the temperature change and the gradient of the last G2P agree with
    the FP64 restatement."""
    sc = scenes.thermal_block()
    gpu = run_gpu(sc, 2)
    ref = run_oracle(sc, 2)
    assert rel_l2(_dT(gpu._get_particles("temp"), sc), _dT(ref.pfield("temp"), sc)) <= STEP_TOL
    assert rel_l2(gpu._get_particles("tempgrad"), ref.pfield("tempgrad")) <= STEP_TOL


@pytest.mark.parametrize("name", ["thermal_block", "thermal_2d"])
def test_thermal_golden(gpu_lib, name):
    """30-40 steps against the reference's own output (harness sequence), 3D and 2D."""
    gold = np.load(os.path.join(GOLDEN, name + ".npz"))
    make, steps, _ = make_golden.CASES[name]
    sc = make()
    gpu = run_gpu(sc, int(gold["steps"]))
    ids = gold["ids"]
    got = gpu._get_particles("temp")[ids]
    assert rel_l2(got - sc.temp[ids], gold["temp"] - sc.temp[ids]) <= MANY_STEP_TOL
    assert rel_l2(gpu._get_particles("tempgrad")[ids], gold["tempgrad"]) <= MANY_STEP_TOL
    for f in ("vel", "stress"):
        a, b = gpu._get_particles(f)[ids], gold[f]
        if np.linalg.norm(b) == 0:
            assert np.max(np.abs(a)) < 1e-9
        else:
            assert rel_l2(a, b) <= MANY_STEP_TOL


def test_thermal_temperatures_reset_between_steps(gpu_lib, oracle_built):
    """The pattern of Examples/thermalTest.py: the script sets the hot and cold zones'
    temperatures again after every step; the GPU takes the values between steps."""
    from graphyt_gb300 import graphyt
    from oracle.oracle import Oracle
    sc = scenes.thermal_block()
    hot = np.nonzero(sc.temp == 100.0)[0]
    cold = np.nonzero(sc.temp == 50.0)[0]
    gpu = graphyt.from_scene(sc)
    ref = Oracle(sc, "port")
    dt = gpu.dt
    for k in range(20):
        gpu.iterate_GPU(k * dt, k)
        ref.step()
        gpu.mpts.setTemps(hot, 100.0)
        gpu.mpts.setTemps(cold, 50.0)
        ref.set_temps(hot, np.full(hot.size, 100.0))
        ref.set_temps(cold, np.full(cold.size, 50.0))
    gpu.Synchronise()
    a, b = gpu.mpts.getTemperatureArr(), ref.pfield("temp")
    assert np.array_equal(a[hot], b[hot]) and np.array_equal(a[cold], b[cold])
    assert rel_l2(a - sc.temp, b - sc.temp) <= MANY_STEP_TOL
    assert np.abs(b - sc.temp).max() > 1.0


def test_thermal_set_after_initialize_enables_conduction(gpu_lib, oracle_built):
    """Temperatures first set after the solver exists start the conduction terms; until then
    every temperature stays at zero and no gradient forms."""
    from graphyt_gb300 import graphyt
    from oracle.oracle import Oracle
    sc = scenes.thermal_block()
    T = sc.temp.copy()
    sc.temp = np.zeros(sc.n)
    gpu = graphyt.from_scene(sc)
    ref = Oracle(sc, "port")
    dt = gpu.dt
    for k in range(3):
        gpu.iterate_GPU(k * dt, k)
        ref.step()
    assert np.all(gpu.mpts.getTemperatureArr() == 0.0)
    assert np.all(gpu._get_particles("tempgrad") == 0.0)
    nz = np.nonzero(T)[0]
    gpu.mpts.setTemps(nz, T[nz])
    ref.set_temps(nz, T[nz])
    for k in range(3, 12):
        gpu.iterate_GPU(k * dt, k)
        ref.step()
    gpu.Synchronise()
    assert rel_l2(gpu._get_particles("temp") - T, ref.pfield("temp") - T) <= MANY_STEP_TOL


def test_thermal_two_bodies(gpu_lib, oracle_built):
    """Conduction is body-agnostic (centre-of-mass nodes), rigid particles count with m = 1:
    two blocks in contact, the second rigid, with a temperature on part of each."""
    sc = scenes.two_blocks(rigid_second=True)
    y = sc.pos[:, 1]
    sc.temp = np.where(y > np.median(y), 80.0, 0.0) + np.where(sc.obj == sc.obj.max(), 20.0, 0.0)
    gpu = run_gpu(sc, 15)
    ref = run_oracle(sc, 15)
    assert rel_l2(gpu._get_particles("temp") - sc.temp, ref.pfield("temp") - sc.temp) <= MANY_STEP_TOL
    assert rel_l2(gpu._get_particles("vel"), ref.pfield("vel")) <= MANY_STEP_TOL


def test_thermal_checkpoint_resume(gpu_lib, tmp_path):
    """The snapshot carries the temperatures and gradients."""
    from graphyt_gb300 import graphyt
    sc = scenes.thermal_block()
    a = graphyt.from_scene(sc)
    dt = a.dt
    for k in range(8):
        a.iterate_GPU(k * dt, k)
    path = str(tmp_path / "state.bin")
    a.save(path)
    for k in range(8, 16):
        a.iterate_GPU(k * dt, k)
    a.Synchronise()
    b = graphyt.from_scene(sc)
    b.load(path)
    for k in range(8, 16):
        b.iterate_GPU(k * dt, k)
    b.Synchronise()
    ta, tb = a._get_particles("temp"), b._get_particles("temp")
    assert rel_l2(tb - sc.temp, ta - sc.temp) < 1e-5


def test_thermal_handle_rejects_state_without_temperatures(gpu_lib, tmp_path):
    """A state saved by a run without heat conduction does not load into a handle that carries
    temperatures (it would keep its own temperatures and step on unlike the saved run); the
    handle is left as it was."""
    from graphyt_gb300 import _lib, graphyt
    sc = scenes.thermal_block()
    cold = sc.__class__(**{**sc.__dict__})
    cold.temp = np.zeros_like(sc.temp)
    a = graphyt.from_scene(cold)
    dt = a.dt
    for k in range(3):
        a.iterate_GPU(k * dt, k)
    path = str(tmp_path / "cold.bin")
    a.save(path)
    b = graphyt.from_scene(sc)
    b.iterate_GPU(0.0, 0)
    before = b._get_particles("temp")
    with pytest.raises(_lib.GraphytGPUError):
        b.load(path)
    assert np.array_equal(b._get_particles("temp"), before)


def test_no_temperature_no_conduction(gpu_lib):
    """With every temperature zero the step runs without the thermal terms and the
    temperature getters report zeros; the first nonzero temperature adds one launch, the
    clear of the thermal node fields, to every step (the single-body P2G and G2P kernels run
    their heat conduction variants)."""
    from graphyt_gb300 import graphyt
    lib = gpu_lib
    sc = scenes.tiny_block(model=1)
    gpu = graphyt.from_scene(sc)
    dt = gpu.dt

    def launches(k0, k1):
        gpu.Synchronise()
        n0 = lib.gy_kernel_launches()
        for k in range(k0, k1):
            gpu.iterate_GPU(k * dt, k)
        gpu.Synchronise()
        return lib.gy_kernel_launches() - n0

    launches(0, 3)
    plain = launches(3, 6)
    assert np.all(gpu._get_particles("temp") == 0.0)
    assert np.all(gpu._get_particles("tempgrad") == 0.0)
    gpu.mpts.setTemps(np.arange(sc.n // 2), 10.0)
    warm = launches(6, 9)
    assert warm == plain + 3
    assert np.any(gpu._get_particles("tempgrad") != 0.0)


def test_thermal_between_sorts(gpu_lib, oracle_built):
    """With the particles re-ordered only every third step, the thermal kernels walk the
    unsorted runs of cell blocks and give the same temperatures."""
    sc = scenes.thermal_block()
    gpu = run_gpu(sc, 12, options=dict(sort_every=3))
    ref = run_oracle(sc, 12)
    assert rel_l2(_dT(gpu._get_particles("temp"), sc), _dT(ref.pfield("temp"), sc)) <= MANY_STEP_TOL


@pytest.mark.parametrize("make", [lambda: scenes.thermal_block(), lambda: scenes.thermal_2d()])
def test_thermal_p2g_lane_variants_agree(gpu_lib, make):
    """The heat conduction variants of the two P2G lane mappings (three z-plane lanes or nine
    x-column lanes per run of equal cell) form the same sums in another order: temperatures,
    gradients, velocity and stress agree to FP32 summation order, sorting every step and
    between sorts, in 3D and 2D."""
    sc = make()
    for sort_every in (1, 3):
        a = run_gpu(sc, 20, options=dict(p2g_lanes=3, sort_every=sort_every))
        b = run_gpu(sc, 20, options=dict(p2g_lanes=9, sort_every=sort_every))
        assert rel_l2(_dT(a._get_particles("temp"), sc), _dT(b._get_particles("temp"), sc)) < 1e-5
        for f in ("tempgrad", "vel", "stress"):
            assert rel_l2(a._get_particles(f), b._get_particles(f)) < 1e-5, (f, sort_every)
