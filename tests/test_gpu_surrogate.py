"""The learned Drucker-Prager surrogate in the step: training pairs logged by the exact return
mapping, the MLP trained on them on the tensor cores, and surrogate runs against plain runs.

The surrogate has no reference counterpart; its oracle is the plain GPU return mapping
(ConstitutiveModels.cpp:238-429), which the FP64 restatement pins elsewhere."""
import numpy as np
import pytest

from graphyt_gb300 import graphyt, scenes
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

STEPS_LOG = 400
STEPS_RUN = 250


def _run(sc, steps, surrogate=None, tol=1e-4):
    s = graphyt.from_scene(sc)
    if surrogate is not None:
        s.set_surrogate(True, params=surrogate, tol=tol)
    dt = s.dt
    for k in range(steps):
        s.iterate_GPU(k * dt, k)
    s.Synchronise()
    return s


@pytest.fixture(scope="module")
def trained(gpu_lib):
    """The coarse Brazilian disc (11,392 particles) run with the exact return mapping for 400
    steps while logging every yielding particle's return, then a surrogate trained on the log."""
    sc = scenes.brazilian_disc(scale=0.1)
    s = graphyt.from_scene(sc)
    s.dp_log_begin(cap=4_000_000, every=1)
    dt = s.dt
    for k in range(STEPS_LOG):
        s.iterate_GPU(k * dt, k)
    s.Synchronise()
    x, y = s.dp_log_read()
    loss0 = s.train_surrogate(steps=1, batch=4096, lr=1e-3, seed=0)
    loss = s.train_surrogate(steps=4000, batch=4096, lr=1e-3, seed=0)
    params = s.surrogate_params()
    s.close()
    return dict(scene=sc, x=x, y=y, loss0=loss0, loss=loss, params=params)


def test_logged_returns_land_on_the_yield_surface(trained):
    """Every logged pair is an exact Drucker-Prager return: the elastic trial stress from the
    logged strain increment and previous stress, plus the logged correction, lies on the
    softened yield surface F = 0 (ConstitutiveModels.cpp:321-344) to FP32 rounding, with a
    non-negative plastic strain increment; cohesion and friction angle are the disc's."""
    x, y = trained["x"].astype(np.float64), trained["y"].astype(np.float64)
    assert len(x) > 1000
    mat = trained["scene"].materials[0]
    K, G, coh, ecr = mat["bulkMod"], mat["shearMod"], mat["cohesion"], mat["criticalStrain"]
    assert np.all(x[:, 14] == np.float32(coh)) and np.all(x[:, 15] == np.float32(mat["phi"]))
    de, s0, eq0 = x[:, :6], x[:, 6:12], x[:, 12]
    vol = 0.3333 * de[:, :3].sum(axis=1)
    t = s0.copy()
    t[:, :3] += 2.0 * G * (de[:, :3] - vol[:, None]) + 3.0 * K * vol[:, None]
    t[:, 3:] += 2.0 * G * de[:, 3:]
    s = t + y[:, :6]
    eq = eq0 + y[:, 6]
    assert np.all(y[:, 6] >= 0.0)
    phi = np.deg2rad(mat["phi"]) * 3.14159 / np.pi
    eta = 6.0 * np.sin(phi) / (np.sqrt(3.0) * (3.0 - np.sin(phi)))
    xi = 6.0 * np.cos(phi) / (np.sqrt(3.0) * (3.0 - np.sin(phi)))
    I1 = s[:, :3].mean(axis=1)
    dev = s[:, :3] - I1[:, None]
    J2 = 0.5 * ((dev ** 2).sum(axis=1) + 2.0 * (s[:, 3:] ** 2).sum(axis=1))
    c = np.maximum(coh - eq * coh / ecr, coh / 10.0)
    F = np.sqrt(J2) + eta * I1 - xi * c
    scale = np.abs(t).max(axis=1) + coh
    assert np.all(np.abs(F) <= 2e-5 * scale), np.abs(F / scale).max()


def test_surrogate_training_reduces_loss(trained):
    """Training on the logged returns lowers the normalised mean squared error at least
    tenfold from the first step's."""
    assert trained["loss"] < 0.1 * trained["loss0"], (trained["loss0"], trained["loss"])


def test_surrogate_run_matches_plain_run(trained):
    """With the surrogate on (tolerance 1e-4 x cohesion on the yield residual and on the
    distance to the flow-rule stress of the predicted multiplier), the disc after 250 steps
    has the plain run's stress, velocity and plastic strain to 1e-3 (relative L2; the plain
    return mapping judges the surrogate's error), and every deferred particle was either kept
    or handed back to the exact mapping."""
    sc = trained["scene"]
    plain = _run(sc, STEPS_RUN)
    surr = _run(sc, STEPS_RUN, surrogate=trained["params"], tol=1e-4)
    counts = surr.surrogate_counts()
    assert counts["kept"] + counts["fallback"] > 0
    for f in ("stress", "vel", "eqps"):
        err = rel_l2(surr._get_particles(f), plain._get_particles(f))
        assert err <= 1e-3, (f, err, counts)


def test_surrogate_predictions_kept_everywhere(trained):
    """With the checks opened wide the deferred particles take the MLP's return (those with a
    negative predicted plastic strain increment still fall back): the run stays finite and
    its stress stays within 5e-2 of the plain run -- the trained network's own accuracy over
    250 steps."""
    sc = trained["scene"]
    plain = _run(sc, STEPS_RUN)
    surr = _run(sc, STEPS_RUN, surrogate=trained["params"], tol=1e30)
    counts = surr.surrogate_counts()
    assert counts["kept"] > 0.9 * (counts["kept"] + counts["fallback"]), counts
    s = surr._get_particles("stress")
    assert np.all(np.isfinite(s))
    assert rel_l2(s, plain._get_particles("stress")) <= 5e-2, (rel_l2(s, plain._get_particles("stress")), counts)
