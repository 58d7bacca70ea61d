"""Seeded synthetic scenes for the explicit GIMP MPM step.

Graphyt scripts build geometry with the external ``pyck`` packer (e.g.
``test/test_2d_impact_elastic.py:36-54``), which is not available.  This module stands
in for it: particles sit on a cubic lattice of spacing ``psep`` whose first point is at
``lower + psep/2`` in every shape, with objectID / material fields per shape, the same
fields ``MaterialPoints::addPyckIntField`` consumes (``MaterialPoints.cpp:32-54``).

A :class:`Scene` is plain numpy data; both the GPU solver (through the
``graphyt_gb300.graphyt`` surface) and the CPU oracle are built from the same scene, so
parity runs see bit-identical inputs.  Particle order is shuffled with
``numpy.random.default_rng(seed)`` so that the sort has real work to do.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence

import numpy as np

# BCTypes::function values (BoundaryConditions.hpp:6-77)
BC = dict(none=0, grid_vx=1, grid_vy=2, grid_vz=3, grid_vx_vy=11, grid_vx_vz=12, grid_vy_vz=13,
          grid_vx_vy_vz=18, mp_vx=33, mp_vy=34, mp_vz=35, mp_fx=37, mp_fy=38, mp_fz=39,
          mp_vx_vy=40, mp_fx_fy=43, mp_stress_xx_yy=63, mp_vxsin=65, mp_vysin=66, mp_syysin=67)

# MaterialModels defaults (MaterialModels.cpp:4-26)
MATERIAL_DEFAULTS = dict(bulkMod=1e7, shearMod=5000.0, density=1000.0, isRigid=0, viscosity=1.0,
                         thermalConductivity=391.0, specificHeatCapacity=385.2, yieldStress=1e7,
                         phi=40.0, psi=10.0, cohesion=100000.0, criticalStrain=0.01, isDamage=0,
                         damageModel=1, Cg=586.52, damageM=9.0, damageK=5.39e36, turbStress=1e10,
                         model=1)


def material(**kw) -> Dict:
    m = dict(MATERIAL_DEFAULTS)
    for k, v in kw.items():
        if k not in m:
            raise KeyError(f"unknown material property {k!r}")
        m[k] = v
    return m


@dataclasses.dataclass
class Scene:
    name: str
    L: List[float]
    cellsize: float
    psep: float
    pos: np.ndarray                    # (N, 3) float64
    mat: np.ndarray                    # (N,) int32
    obj: np.ndarray                    # (N,) int32
    materials: List[Dict]
    gravity: List[float] = dataclasses.field(default_factory=lambda: [0.0, 0.0, 0.0])
    damping: float = 0.0
    mu: float = 0.0
    CFL: float = 0.1
    tmax: float = 1.0
    dt: Optional[float] = None         # setDt override; None keeps the Solver's CFL dt
    fixed_grid_bcs: int = 0
    vel: Optional[np.ndarray] = None   # (N, 3)
    stress: Optional[np.ndarray] = None  # (N, 6)
    pbc_type: Optional[np.ndarray] = None  # (N,)
    pbc_val: Optional[np.ndarray] = None   # (N, 4)
    hold: Optional[np.ndarray] = None      # (N,) bool
    node_bc_type: Optional[np.ndarray] = None  # (Nn,)
    node_bc_val: Optional[np.ndarray] = None   # (Nn, 4)
    temp: Optional[np.ndarray] = None          # (N,) temperature (MaterialPoints::setTemp)
    flaw: Optional[np.ndarray] = None          # (N,) Grady-Kipp activation strain scale (1: reference)
    inst: Optional[np.ndarray] = None          # (N,) instance index, for a batch of instances
    instances: Optional[List["Instance"]] = None

    @property
    def is3D(self) -> bool:
        return self.L[2] > 0.0

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def dims(self):
        nx = int(1.0 + self.L[0] / self.cellsize)
        ny = int(1.0 + self.L[1] / self.cellsize)
        nz = int(1.0 + self.L[2] / self.cellsize)
        return nx, ny, nz

    def num_nodes(self) -> int:
        nx, ny, nz = self.dims()
        return nx * ny * nz

    def node_positions(self) -> np.ndarray:
        """Node coordinates i*h, laid out i + j*Nx + k*Nx*Ny (Nodes.cpp:77-139)."""
        nx, ny, nz = self.dims()
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        h = self.cellsize
        return np.stack([i.ravel() * h, j.ravel() * h, k.ravel() * h], axis=1)


def lattice_box(lower, upper, psep):
    """Lattice points lower + psep/2 + i*psep strictly inside [lower, upper)."""
    axes = []
    for lo, hi in zip(lower, upper):
        if hi <= lo:
            axes.append(np.array([lo]))
            continue
        n = int(math.floor((hi - lo) / psep + 1e-9))
        axes.append(lo + psep / 2 + psep * np.arange(n))
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def lattice_cylinder_z(center, radius, z0, z1, psep):
    """Lattice points of a cylinder whose axis is parallel to z."""
    lo = [center[0] - radius, center[1] - radius, z0]
    hi = [center[0] + radius, center[1] + radius, z1]
    p = lattice_box(lo, hi, psep)
    r2 = (p[:, 0] - center[0]) ** 2 + (p[:, 1] - center[1]) ** 2
    return p[r2 <= radius * radius]


def _finish(scene: Scene, seed: int) -> Scene:
    n = scene.n
    if scene.vel is None:
        scene.vel = np.zeros((n, 3))
    if scene.stress is None:
        scene.stress = np.zeros((n, 6))
    if scene.pbc_type is None:
        scene.pbc_type = np.zeros(n, np.int32)
    if scene.pbc_val is None:
        scene.pbc_val = np.zeros((n, 4))
    if scene.hold is None:
        scene.hold = np.zeros(n, bool)
    if scene.temp is None:
        scene.temp = np.zeros(n)
    nn = scene.num_nodes()
    if scene.node_bc_type is None:
        scene.node_bc_type = np.zeros(nn, np.int32)
    if scene.node_bc_val is None:
        scene.node_bc_val = np.zeros((nn, 4))
    if seed is not None:
        perm = np.random.default_rng(seed).permutation(n)
        for f in ("pos", "mat", "obj", "vel", "stress", "pbc_type", "pbc_val", "hold", "temp", "inst", "flaw"):
            if getattr(scene, f) is not None:
                setattr(scene, f, np.ascontiguousarray(getattr(scene, f)[perm]))
    scene.pos = np.ascontiguousarray(scene.pos, np.float64)
    scene.mat = np.ascontiguousarray(scene.mat, np.int32)
    scene.obj = np.ascontiguousarray(scene.obj, np.int32)
    scene.pbc_type = np.ascontiguousarray(scene.pbc_type, np.int32)
    scene.node_bc_type = np.ascontiguousarray(scene.node_bc_type, np.int32)
    return scene


def weibull_flaws(scene: Scene, seed: int = 0) -> Scene:
    """Per-particle flaw activation strains drawn from the Weibull law, seeded.

    Grady-Kipp flaws are a Poisson population whose number per unit volume with activation
    strain below e is k e^m, so the weakest flaw of a particle of volume V activates at the
    strain e with P(e_w > e) = exp(-V k e^m): e_w = (V k)^(-1/m) (-ln U)^(1/m) for uniform U.
    The reference uses the deterministic (V k)^(-1/m) (DamageModels.cpp:102-103), the case
    -ln U = 1.  The draw is stored as the scale w = (-ln U)^(1/m), applied to the e_min the
    step computes from the particle's current volume.  Particles of materials without
    Grady-Kipp damage keep w = 1."""
    rng = np.random.default_rng(seed)
    u = 1.0 - rng.random(scene.n)  # in (0, 1]
    m = np.array([float(mt["damageM"]) if mt["isDamage"] and mt["damageModel"] == 1 else 0.0
                  for mt in scene.materials])[scene.mat]
    w = np.ones(scene.n)
    on = m > 0
    w[on] = (-np.log(u[on])) ** (1.0 / m[on])
    scene.flaw = w
    return scene


# ------------------------------------------------------------------------------------------
# named workloads

def elastic_cube(variant: str = "particle", scale: int = 1, seed: int = 0, offset=None) -> Scene:
    """Elastic cube compression: 1 m periodic domain, cellsize 0.05/scale, psep half of it,
    a 0.5 m cube centred in the domain (20^3 = 8000 particles at scale 1), K 1e7, G 5e6,
    rho 1000, no gravity, dt = 0.3*dx/sqrt((K+4G/3)/rho) through setDt.

    variant "nodal":    grid_vz on the node layer touching the cube top (-0.1 m/s) and
                         bottom (0); these bodies are empty in the reference, so the cube stays
                         at rest (bug-compatible run).
    variant "fixed":    the same nodal BCs with fixed_grid_bcs=1 (working z BCs).
    variant "particle": mp_vz on the top particle layer (-0.1) and bottom layer (0).

    offset shifts the whole lattice.  The centred lattice puts the cube's outer particles
    exactly on the edge of the GIMP support of the next node layer; there the reference's
    own result is discontinuous in the particle position (a node reached with a vanishing
    weight contributes a finite strain rate through f/m), so long runs are ill-conditioned
    in FP64 as well.  A shift of a few millimetres removes that degeneracy.
    """
    h = 0.05 / scale
    psep = h / 2
    pos = lattice_box([0.25, 0.25, 0.25], [0.75, 0.75, 0.75], psep)
    if offset is not None:
        pos = pos + np.asarray(offset, np.float64)
    n = len(pos)
    K, G, rho = 1e7, 5e6, 1000.0
    sc = Scene("elastic_cube_" + variant, [1.0, 1.0, 1.0], h, psep, pos, np.zeros(n, np.int32),
               np.zeros(n, np.int32), [material(bulkMod=K, shearMod=G, density=rho, model=1)])
    sc.dt = 0.3 * h / math.sqrt((K + 4.0 * G / 3.0) / rho)
    sc.tmax = 1000 * sc.dt
    if variant == "particle":
        ztop, zbot = pos[:, 2].max(), pos[:, 2].min()
        sc.pbc_type = np.zeros(n, np.int32)
        sc.pbc_val = np.zeros((n, 4))
        top = np.isclose(pos[:, 2], ztop)
        bot = np.isclose(pos[:, 2], zbot)
        sc.pbc_type[top | bot] = BC["mp_vz"]
        sc.pbc_val[top, 0] = -0.1
    else:
        nodes = sc.node_positions()
        nn = len(nodes)
        sc.node_bc_type = np.zeros(nn, np.int32)
        sc.node_bc_val = np.zeros((nn, 4))
        inside = ((nodes[:, 0] >= 0.25 - 1e-9) & (nodes[:, 0] <= 0.75 + 1e-9) &
                  (nodes[:, 1] >= 0.25 - 1e-9) & (nodes[:, 1] <= 0.75 + 1e-9))
        top = inside & np.isclose(nodes[:, 2], 0.75)
        bot = inside & np.isclose(nodes[:, 2], 0.25)
        sc.node_bc_type[top | bot] = BC["grid_vz"]
        sc.node_bc_val[top, 0] = -0.1
        sc.fixed_grid_bcs = 1 if variant == "fixed" else 0
    return _finish(sc, seed)


def dam_break(scale: float = 1.0, height: float = 0.765, seed: int = 0, walls: bool = True,
              width: float = 2.0) -> Scene:
    """3D Newtonian dam break: domain 4 x width x 2 m (width 2 by default), cellsize
    0.01/scale, psep half of it.
    Water (K 2e6, viscosity 1e-3, rho 1000) fills x in [2h, 2h+1.0], y in [2h, width-2h],
    z in [2h, 2h+height] against the x=0 wall; gravity -9.81 in z; CFL 0.3 with the
    Solver's own dt formula (Solver.cpp:32).  At scale 1 and the default height this is
    200 x 392 x 153 = 11,997,600 particles.  With walls=True every node within two cells
    of a face carries grid_vx_vy_vz = 0 with fixed_grid_bcs=1 (the reference's
    grid_vx_vy_vz body is empty, Grid.cpp:1050-1052)."""
    h = 0.01 / scale
    psep = h / 2
    L = [4.0, float(width), 2.0]
    w = 2 * h
    pos = lattice_box([w, w, w], [w + 1.0, L[1] - w, w + height], psep)
    n = len(pos)
    sc = Scene("dam_break", L, h, psep, pos, np.zeros(n, np.int32), np.zeros(n, np.int32),
               [material(bulkMod=2e6, viscosity=1e-3, density=1000.0, shearMod=0.0, model=2)])
    sc.gravity = [0.0, 0.0, -9.81]
    sc.CFL = 0.3
    sc.tmax = 1.0
    if walls:
        nx, ny, nz = sc.dims()
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        near = ((i <= 2) | (i >= nx - 3) | (j <= 2) | (j >= ny - 3) | (k <= 2) | (k >= nz - 3))
        sc.node_bc_type = np.where(near, BC["grid_vx_vy_vz"], 0).astype(np.int32)
        sc.node_bc_val = np.zeros((nx * ny * nz, 4))
        sc.fixed_grid_bcs = 1
    return _finish(sc, seed)


def brazilian_disc(scale: float = 1.0, seed: int = 0, platen_speed: float = 0.5, shift: bool = True,
                   weibull_seed: Optional[int] = None) -> Scene:
    """3D Brazilian disc: a Drucker-Prager + Grady-Kipp cylinder (radius 0.05 m, thickness
    0.02 m, axis along z) squeezed along y by two rigid platens at +/-platen_speed.
    cellsize 5e-4/scale, psep half of it.  DP: K 3e10, G 2e10, rho 2600, cohesion 1e7,
    friction 30 deg, dilatancy 0, critical strain 0.01.  GK: m 9, k 5e32, Cg = 0.4 x the
    P-wave speed (1867.40 m/s).  objectIDs: disc 1, top platen 2, bottom platen 3 (the
    layout of Examples/brazillian3D.py:31-108).  At scale 1 this is about 10 M particles.
    The reference's Grady-Kipp flaw threshold is the deterministic e_min = (V k)^(-1/m)
    (DamageModels.cpp:102-103); weibull_seed draws per-particle Weibull activation strains
    instead (weibull_flaws).

    shift moves the whole lattice by (0.0931, 0.0517, 0.0713) psep.  Unshifted, particles sit
    exactly on the reference's quarter-cell binning boundaries (TimeIntegration.cpp:111-113),
    where its own FP64 rounding decides which cell -- and so which body slot of a contact
    node (Extrapolation.cpp:191-198) -- a particle lands in."""
    h = 5e-4 / scale
    psep = h / 2
    R, T = 0.05, 0.02
    margin = 8 * h
    Lx = 2 * R + 2 * margin
    Ly = 2 * R + 2 * margin + 4 * h + 2 * 4 * h
    Lz = T + 2 * margin
    L = [round(Lx / h) * h, round(Ly / h) * h, round(Lz / h) * h]
    cx, cy = L[0] / 2, L[1] / 2
    z0 = margin
    disc = lattice_cylinder_z([cx, cy], R, z0, z0 + T, psep)
    pw = 4 * h  # platen thickness
    half = 0.25 * R
    top = lattice_box([cx - half, cy + R + psep, z0], [cx + half, cy + R + psep + pw, z0 + T], psep)
    bot = lattice_box([cx - half, cy - R - psep - pw, z0], [cx + half, cy - R - psep, z0 + T], psep)
    pos = np.concatenate([disc, top, bot])
    if shift:
        pos = pos + np.array([0.0931, 0.0517, 0.0713]) * psep
    mat = np.concatenate([np.zeros(len(disc)), np.ones(len(top)), np.ones(len(bot))]).astype(np.int32)
    obj = np.concatenate([np.full(len(disc), 1), np.full(len(top), 2), np.full(len(bot), 3)]).astype(np.int32)
    K, G, rho = 3e10, 2e10, 2600.0
    cp = math.sqrt((K + 4.0 * G / 3.0) / rho)
    rock = material(bulkMod=K, shearMod=G, density=rho, cohesion=1e7, phi=30.0, psi=0.0,
                    criticalStrain=0.01, isDamage=1, damageModel=1, Cg=0.4 * cp, damageM=9.0,
                    damageK=5e32, model=4)
    platen = material(isRigid=1)
    sc = Scene("brazilian_disc", L, h, psep, pos, mat, obj, [rock, platen])
    sc.CFL = 0.3
    sc.tmax = 1.0
    vel = np.zeros((len(pos), 3))
    vel[obj == 2, 1] = -platen_speed
    vel[obj == 3, 1] = platen_speed
    sc.vel = vel
    sc = _finish(sc, seed)
    return sc if weibull_seed is None else weibull_flaws(sc, weibull_seed)


def tiny_block(seed: int = 0, model: int = 1, n_side: int = 4, cellsize: float = 0.125,
               L=(1.5, 1.5, 1.5), gravity=(0.0, 0.0, -9.81), vel=(0.3, -0.2, 0.1)) -> Scene:
    """A small block for fast parity cases: n_side^3 particles on a 12^3-cell grid."""
    h = cellsize
    psep = h / 2
    lo = np.array([0.5, 0.45, 0.4])
    pos = lattice_box(lo, lo + n_side * psep, psep)
    n = len(pos)
    mats = [material(bulkMod=1e6, shearMod=4e5, density=1200.0, viscosity=0.5, yieldStress=2e3,
                     cohesion=2e3, phi=30.0, psi=10.0, criticalStrain=0.05, model=model)]
    sc = Scene(f"tiny_block_m{model}", list(L), h, psep, pos, np.zeros(n, np.int32),
               np.zeros(n, np.int32), mats)
    sc.gravity = list(gravity)
    sc.CFL = 0.3
    v = np.zeros((n, 3))
    v[:] = vel
    v += 0.05 * np.random.default_rng(seed + 1).standard_normal((n, 3))
    sc.vel = v
    return _finish(sc, seed)


def damage_block(seed: int = 0, n_side: int = 8, weibull_seed: Optional[int] = None) -> Scene:
    """A Drucker-Prager + Grady-Kipp block on a 12^3-cell grid, stretched along x and
    squeezed along z by its initial velocity field so that both the damage growth (tension)
    and the plastic return (compression) act within a few tens of steps."""
    h = 0.125
    psep = h / 2
    lo = np.array([0.45, 0.45, 0.45])
    pos = lattice_box(lo, lo + n_side * psep, psep)
    n = len(pos)
    c = pos.mean(axis=0)
    rock = material(bulkMod=1e6, shearMod=6e5, density=1500.0, cohesion=3e3, phi=30.0, psi=5.0,
                    criticalStrain=0.02, isDamage=1, damageModel=1, Cg=0.05, damageM=9.0,
                    damageK=1e28, model=4)
    sc = Scene("damage_block", [1.5, 1.5, 1.5], h, psep, pos, np.zeros(n, np.int32), np.zeros(n, np.int32),
               [rock])
    sc.CFL = 0.3
    v = np.zeros((n, 3))
    v[:, 0] = 3.0 * (pos[:, 0] - c[0])
    v[:, 2] = -2.0 * (pos[:, 2] - c[2])
    v += 0.02 * np.random.default_rng(seed + 5).standard_normal((n, 3))
    sc.vel = v
    sc = _finish(sc, seed)
    return sc if weibull_seed is None else weibull_flaws(sc, weibull_seed)


def two_blocks(seed: int = 0, speed: float = 1.5, rigid_second: bool = False) -> Scene:
    """Two elastic blocks (objectIDs 1 and 2) approaching along x at +/-speed: the two-body
    contact branch of the nodal solve (Grid.cpp:50-219).  With rigid_second the second block
    is a rigid platen (Grid.cpp:78-105)."""
    h = 0.0625
    psep = h / 2
    a = lattice_box([0.35, 0.40, 0.40], [0.60, 0.65, 0.65], psep)
    b = lattice_box([0.66, 0.40, 0.40], [0.91, 0.65, 0.65], psep)
    pos = np.concatenate([a, b])
    obj = np.concatenate([np.full(len(a), 1), np.full(len(b), 2)]).astype(np.int32)
    mat = np.concatenate([np.zeros(len(a)), np.full(len(b), 1 if rigid_second else 0)]).astype(np.int32)
    mats = [material(bulkMod=2e6, shearMod=1e6, density=1000.0, model=1)]
    if rigid_second:
        mats.append(material(isRigid=1))
    sc = Scene("two_blocks_rigid" if rigid_second else "two_blocks", [1.25, 1.0, 1.0], h, psep, pos, mat, obj, mats)
    sc.CFL = 0.3
    sc.mu = 0.2
    v = np.zeros((len(pos), 3))
    v[obj == 1, 0] = speed
    v[obj == 2, 0] = -speed
    sc.vel = v
    return _finish(sc, seed)


def block_2d(seed: int = 0, model: int = 1, platen: bool = True, shift: bool = True) -> Scene:
    """2D plane-strain block (L[2] = 0) in the layout of the reference's 2D tests
    (test/test_2d_elastic_uniaxial_compression.py): a rock block, optionally under a rigid
    platen moving down at 0.2 m/s, gravity off.  shift moves the lattice by (0.0931, 0.0517)
    psep off the quarter-cell binning boundaries, where the reference's own result depends
    on FP64 rounding (see brazilian_disc)."""
    h = 0.01
    psep = h / 2
    blk = lattice_box([0.05, 0.03, 0.0], [0.15, 0.23, 0.0], psep)
    parts = [blk]
    mat = [np.zeros(len(blk))]
    obj = [np.full(len(blk), 1)]
    if platen:
        pl = lattice_box([0.04, 0.23 + psep, 0.0], [0.16, 0.23 + psep + 3 * psep, 0.0], psep)
        parts.append(pl)
        mat.append(np.ones(len(pl)))
        obj.append(np.full(len(pl), 2))
    pos = np.concatenate(parts)
    if shift:
        pos[:, :2] += np.array([0.0931, 0.0517]) * psep
    mats = [material(bulkMod=3.31e9, shearMod=2.48e9, density=1540.0, yieldStress=2e5, cohesion=1e5, phi=30.0,
                     psi=5.0, model=model)]
    if platen:
        mats.append(material(isRigid=1))
    sc = Scene(f"block_2d_m{model}", [0.3, 0.3, 0.0], h, psep, pos, np.concatenate(mat).astype(np.int32),
               np.concatenate(obj).astype(np.int32), mats)
    sc.CFL = 0.3
    v = np.zeros((len(pos), 3))
    if platen:
        v[sc.obj == 2, 1] = -0.2
    sc.vel = v
    return _finish(sc, seed)


def thermal_block(seed: int = 0, n_side: int = 10, cellsize: float = 0.05, model: int = 1,
                  T_cold: float = 50.0, T_hot: float = 100.0) -> Scene:
    """Heat conduction in a 3D block at rest (the pattern of Examples/thermalTest.py): the
    particles of the lowest fifth in y start at T_cold, the highest fifth at T_hot, the rest
    at 0.  Copper thermal properties (the material defaults, k 391, c 385.2) on an elastic
    body of density 1000; no gravity.  The node temperature is the reference's unnormalised
    sum S T m c (Extrapolation.cpp:281-283)."""
    h = cellsize
    psep = h / 2
    side = n_side * psep
    L = [side + 8 * h, side + 8 * h, side + 8 * h]
    lo = [4 * h + 0.013 * psep, 4 * h + 0.021 * psep, 4 * h + 0.017 * psep]
    pos = lattice_box(lo, [lo[0] + side, lo[1] + side, lo[2] + side], psep)
    n = pos.shape[0]
    y = (pos[:, 1] - lo[1]) / side
    temp = np.zeros(n)
    temp[y < 0.2] = T_cold
    temp[y > 0.8] = T_hot
    sc = Scene(name="thermal_block", L=L, cellsize=h, psep=psep, pos=pos,
               mat=np.zeros(n, np.int32), obj=np.zeros(n, np.int32),
               materials=[material(model=model, bulkMod=1e7, shearMod=5000.0, density=1000.0)],
               gravity=[0.0, 0.0, 0.0], CFL=0.1, temp=temp)
    return _finish(sc, seed)


def thermal_2d(seed: int = 0, cellsize: float = 0.01) -> Scene:
    """2D plate of Examples/thermalTest.py at a reduced size: particles below 30 % of the
    plate height at 50, above 72 % at 100, the rest at 0; copper thermal properties, elastic
    (K 1e7, G 1000) at density 1000 so that a step's temperature change is resolvable in
    FP32; no gravity."""
    h = cellsize
    psep = h / 2
    lo, hi = 6 * h + 0.0931 * psep, 24 * h + 0.0931 * psep
    pos = lattice_box([lo, lo + 0.0517 * psep - 0.0931 * psep, 0.0], [hi, hi, 0.0], psep)
    n = pos.shape[0]
    y = (pos[:, 1] - pos[:, 1].min()) / (pos[:, 1].max() - pos[:, 1].min())
    temp = np.zeros(n)
    temp[y < 0.3] = 50.0
    temp[y > 0.72] = 100.0
    sc = Scene(name="thermal_2d", L=[30 * h, 30 * h, 0.0], cellsize=h, psep=psep, pos=pos,
               mat=np.zeros(n, np.int32), obj=np.zeros(n, np.int32),
               materials=[material(model=1, bulkMod=1e7, shearMod=1000.0, density=1000.0)],
               gravity=[0.0, 0.0, 0.0], CFL=0.1, temp=temp)
    return _finish(sc, seed)


def disk_impact_2d(seed: int = 0) -> Scene:
    """Two elastic disks colliding in 2D, the setting of the reference's
    test/test_2d_impact_elastic.py: domain 0.1 x 0.1 m, cellsize 5e-4, psep half of it, a
    lattice offset by a quarter cell; disk 1 (objectID 1, material 0) centred at
    (0.05, 0.03), disk 2 (objectID 2, material 1) three cells above it, radius 0.005, both
    K 1000, G 500, density 10, moving towards each other at 1.5 m/s; CFL 0.1, gravity off.
    The lattice follows this module's convention, not pyck's, so particle indices differ
    from the reference test's."""
    h = 0.0005
    psep = h / 2
    r = 0.005
    c1 = (0.050, 0.03)
    c2 = (0.050, 0.03 + 0.01 + 3 * h)
    parts, obj, mat = [], [], []
    for k, c in enumerate((c1, c2)):
        lo = [c[0] - r + 0.25 * h, c[1] - r + 0.25 * h, 0.0]
        pts = lattice_box(lo, [c[0] + r + 0.25 * h, c[1] + r + 0.25 * h, 0.0], psep)
        pts = pts[(pts[:, 0] - c[0]) ** 2 + (pts[:, 1] - c[1]) ** 2 <= r * r]
        parts.append(pts)
        obj.append(np.full(len(pts), k + 1))
        mat.append(np.full(len(pts), k))
    pos = np.concatenate(parts)
    mats = [material(bulkMod=1000.0, shearMod=500.0, density=10.0, model=1) for _ in range(2)]
    sc = Scene("disk_impact_2d", [0.10, 0.10, 0.0], h, psep, pos, np.concatenate(mat).astype(np.int32),
               np.concatenate(obj).astype(np.int32), mats)
    sc.CFL = 0.1
    sc.tmax = 5e-3
    v = np.zeros((len(pos), 3))
    v[sc.obj == 1, 1] = 1.5
    v[sc.obj == 2, 1] = -1.5
    sc.vel = v
    return _finish(sc, seed)


# ------------------------------------------------------------------------------------------
# a batch of independent instances in one grid

@dataclasses.dataclass
class Instance:
    """One impact problem of a batch: a sphere (objectID 2, material 0) resting on a
    Drucker-Prager + Grady-Kipp slab (objectID 1, material 1 + index) and moving down at the
    impact speed.  Sizes are in cells of the batch's cellsize; ``box`` is the instance's own
    domain (margin included) and ``origin`` its cell offset in the batch grid."""
    index: int
    target: int
    side: int
    thick: int
    radius: float
    box: tuple
    origin: tuple = (0, 0, 0)
    scale: tuple = (1.0, 1.0, 1.0, 1.0)   # K, G, cohesion, friction angle over the nominal rock
    n: int = 0
    mat: int = 0                          # the slab's material row in its batch


# the rock of the Brazilian disc workload: DP K 3e10, G 2e10, rho 2600, cohesion 1e7,
# friction 30 deg, dilatancy 0, critical strain 0.01; GK m 9, k 5e32, Cg 0.4 x P-wave speed
ROCK = dict(K=3e10, G=2e10, rho=2600.0, cohesion=1e7, phi=30.0)


def _rock(K, G, cohesion, phi, rho=ROCK["rho"]) -> Dict:
    cp = math.sqrt((K + 4.0 * G / 3.0) / rho)
    return material(bulkMod=K, shearMod=G, density=rho, cohesion=cohesion, phi=phi, psi=0.0,
                    criticalStrain=0.01, isDamage=1, damageModel=1, Cg=0.4 * cp, damageM=9.0,
                    damageK=5e32, model=4)


def _impact_count(side: int, thick: int, radius: float) -> int:
    """Particles of a side x side x thick-cell slab (two per cell and axis) plus a sphere of
    the given radius in cells, from the volumes."""
    return 8 * side * side * thick + int(4.0 / 3.0 * math.pi * (2.0 * radius) ** 3)


def _impact_shape(target: int, margin: int):
    """Slab side and thickness (a quarter of the side) and sphere radius (0.15 of the side)
    whose particle count is closest to target."""
    best = None
    for side in range(4, 400):
        thick = max(2, int(round(side / 4)))
        radius = max(1.5, 0.15 * side)
        err = abs(_impact_count(side, thick, radius) - target)
        if best is None or err < best[0]:
            best = (err, side, thick, radius)
    _, side, thick, radius = best
    box = (side + 2 * margin, side + 2 * margin, thick + int(math.ceil(2 * radius)) + 1 + 2 * margin)
    return side, thick, radius, box


def impact_batch_layout(n_inst: int = 256, seed: int = 0, n_min: int = 2000, n_max: int = 200000,
                        margin: int = 5, spread: float = 0.3, shard: Optional[tuple] = None):
    """Instances and the batch grid (cells per axis) without particles.

    Particle counts are drawn log-uniform in [n_min, n_max] and the slab's K, G, cohesion
    and friction angle uniformly within +/-spread of the nominal rock, all from
    numpy.random.default_rng(seed).  The instance boxes are shelf-packed on the x-y plane,
    widest first, in rows along x about as long as the square root of their total area;
    boxes touch, and each keeps ``margin`` empty cells around its content, so neighbouring
    instances never reach a common node (GIMP support spans 1.25 cells) and the periodic
    fold of the outermost three node layers sees no mass.

    shard = (rank, ranks) keeps the instances whose index is rank modulo ranks (the draws are
    those of the whole batch), for one process per GPU each stepping its share."""
    rng = np.random.default_rng(seed)
    targets = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_inst))
    scales = rng.uniform(1.0 - spread, 1.0 + spread, (n_inst, 4))
    insts = []
    for i in range(n_inst):
        if shard is not None and i % shard[1] != shard[0]:
            continue
        side, thick, radius, box = _impact_shape(int(round(targets[i])), margin)
        insts.append(Instance(i, int(round(targets[i])), side, thick, radius, box,
                              scale=tuple(float(v) for v in scales[i])))
    if not insts:
        raise ValueError("the shard holds no instance")
    order = sorted(range(len(insts)), key=lambda i: (-insts[i].box[0], i))
    area = sum(insts[i].box[0] * insts[i].box[1] for i in order)
    row_len = max(insts[order[0]].box[0], int(math.ceil(math.sqrt(area))))
    x = y = depth = width = 0
    for i in order:
        b = insts[i].box
        if x + b[0] > row_len:
            y, x, depth = y + depth, 0, 0
        insts[i].origin = (x, y, 0)
        x += b[0]
        depth = max(depth, b[1])
        width = max(width, x)
    dims = (width, y + depth, max(inst.box[2] for inst in insts))
    return insts, dims


def _impact_particles(inst: Instance, h: float, margin: int):
    """Lattice points of the slab and the sphere in the instance's own frame (a shift of
    (0.0931, 0.0517, 0.0713) psep keeps them off the quarter-cell binning boundaries).  The
    sphere's lowest layer sits one psep above the slab's top layer."""
    psep = h / 2
    m = margin * h
    side, thick = inst.side * h, inst.thick * h
    slab = lattice_box([m, m, m], [m + side, m + side, m + thick], psep)
    r = inst.radius * h
    cx = cy = m + side / 2
    z0 = m + thick
    ball = lattice_box([cx - r, cy - r, z0], [cx + r, cy + r, z0 + 2 * r], psep)
    cz = z0 + r
    ball = ball[((ball[:, 0] - cx) ** 2 + (ball[:, 1] - cy) ** 2 + (ball[:, 2] - cz) ** 2) <= r * r]
    shift = np.array([0.0931, 0.0517, 0.0713]) * psep
    return slab + shift, ball + shift


def impact_batch(n_inst: int = 256, seed: int = 0, n_min: int = 2000, n_max: int = 200000,
                 cellsize: float = 0.01, speed: float = 5.0, margin: int = 5,
                 shard: Optional[tuple] = None) -> Scene:
    """A batch of independent 3D impact problems advanced as one grid: in each instance a
    sphere dropped at ``speed`` onto a Drucker-Prager + Grady-Kipp slab (see
    :func:`impact_batch_layout` for the draws and the packing).  The sphere is elastic with
    the nominal rock's K, G and density; gravity -9.81 in z; every instance steps with the
    batch's dt, the Solver's CFL 0.3 formula over all materials (Solver.cpp:15-32).  At the
    defaults this is 256 instances and about 11 M particles.  ``scene.inst`` holds each
    particle's instance and ``scene.instances`` the layout; ``shard`` as in
    :func:`impact_batch_layout`."""
    h = cellsize
    psep = h / 2
    insts, dims = impact_batch_layout(n_inst, seed, n_min, n_max, margin, shard=shard)
    materials = [material(bulkMod=ROCK["K"], shearMod=ROCK["G"], density=ROCK["rho"], model=1)]
    pos, mat, obj, inst_of, vel = [], [], [], [], []
    for inst in insts:
        slab, ball = _impact_particles(inst, h, margin)
        off = np.array(inst.origin, np.float64) * h
        inst.n = len(slab) + len(ball)
        sK, sG, sc_, sphi = inst.scale
        inst.mat = len(materials)
        materials.append(_rock(ROCK["K"] * sK, ROCK["G"] * sG, ROCK["cohesion"] * sc_, ROCK["phi"] * sphi))
        pos += [slab + off, ball + off]
        mat += [np.full(len(slab), inst.mat), np.zeros(len(ball))]
        obj += [np.full(len(slab), 1), np.full(len(ball), 2)]
        inst_of.append(np.full(inst.n, inst.index))
        v = np.zeros((inst.n, 3))
        v[len(slab):, 2] = -speed
        vel.append(v)
    sc = Scene("impact_batch", [dims[0] * h, dims[1] * h, dims[2] * h], h, psep, np.concatenate(pos),
               np.concatenate(mat).astype(np.int32), np.concatenate(obj).astype(np.int32), materials)
    sc.gravity = [0.0, 0.0, -9.81]
    sc.CFL = 0.3
    sc.tmax = 1.0
    # the whole batch's dt (every shard steps with it): the nominal rock scaled by the
    # largest K factor drawn, over the common density
    maxK = ROCK["K"] * max(1.0, max(_batch_scales(n_inst, seed, n_min, n_max)[:, 0]))
    sc.dt = sc.CFL * (h / math.sqrt(maxK / ROCK["rho"]))
    sc.vel = np.concatenate(vel)
    sc.inst = np.concatenate(inst_of).astype(np.int32)
    sc.instances = insts
    return _finish(sc, seed)


def _batch_scales(n_inst, seed, n_min, n_max, spread: float = 0.3):
    """The material factors of every instance of the whole batch (the draws of
    :func:`impact_batch_layout`)."""
    rng = np.random.default_rng(seed)
    rng.uniform(math.log(n_min), math.log(n_max), n_inst)
    return rng.uniform(1.0 - spread, 1.0 + spread, (n_inst, 4))


def batch_instance(batch: Scene, index: int) -> Scene:
    """Instance ``index`` of a batch as a problem of its own: its particles in the batch's
    order, moved to the instance's own domain (the box at the origin), materials [sphere,
    this slab], the batch's dt and gravity."""
    inst = next(i for i in batch.instances if i.index == index)
    sel = np.nonzero(batch.inst == index)[0]
    h = batch.cellsize
    pos = batch.pos[sel] - np.array(inst.origin, np.float64) * h
    mat = np.where(batch.mat[sel] == 0, 0, 1).astype(np.int32)
    sc = Scene(f"impact_instance_{index}", [b * h for b in inst.box], h, batch.psep, pos, mat,
               batch.obj[sel].copy(), [batch.materials[0], batch.materials[inst.mat]])
    sc.gravity = list(batch.gravity)
    sc.CFL = batch.CFL
    sc.tmax = batch.tmax
    sc.dt = batch.dt
    sc.vel = batch.vel[sel].copy()
    return _finish(sc, None)


# ---- independent problems packed into one grid --------------------------------------------
@dataclasses.dataclass
class PackedInstance:
    """One problem of a packed batch: ``box`` its cells per axis (its own domain plus the
    margin on each side in x and y), ``origin`` the box's cell offset in the batch grid,
    ``first`` / ``n`` its slice of the batch's particles (in insertion order) and ``mat0`` /
    ``nmat`` its rows of the batch's material list."""
    index: int
    name: str
    box: tuple
    origin: tuple
    shift: tuple
    first: int
    n: int
    mat0: int
    nmat: int


def pack_scenes(scenes_: Sequence[Scene], margin: int = 3) -> Scene:
    """Independent problems advanced as one grid (one launch per kernel for all of them).

    Every scene keeps its own domain as a box of the batch grid, ``margin`` empty cells on each
    side in x and y (no GIMP stencil, 1.25 cells, and no body window, 2 cells, reaches from
    one box into the next), the boxes shelf-packed on the x-y plane as in
    :func:`impact_batch_layout`.  Particles, their fields and node BCs move with their box; the
    material lists are concatenated (material indices offset per scene; at most 4096 rows), the
    object ids are kept (the problems never share a node, so they may reuse them).  The scenes
    must agree on the cell size, particle spacing, dimension, gravity, damping, friction, CFL
    and grid-BC mode, and on dt when one sets it; every problem then steps with the batch's dt
    (the Solver formula over all the materials, or the common dt).  The problems' own domain
    walls are not there in the batch, so a problem packs exactly when its particles stay away
    from its domain boundary (the periodic wrap, Solver.cpp's fold of the outermost node
    layers) -- as every scene here does.  ``scene.inst`` gives each particle's problem,
    ``scene.instances`` the layout (:class:`PackedInstance`), ``scene.sources`` the input
    scenes; :func:`unpack_instance` rebuilds one problem alone."""
    if not scenes_:
        raise ValueError("nothing to pack")
    s0 = scenes_[0]
    for sc in scenes_[1:]:
        for attr in ("cellsize", "psep", "damping", "mu", "CFL", "fixed_grid_bcs"):
            if getattr(sc, attr) != getattr(s0, attr):
                raise ValueError(f"pack_scenes: {sc.name} has another {attr} than {s0.name}")
        if list(sc.gravity) != list(s0.gravity) or sc.is3D != s0.is3D or sc.dt != s0.dt:
            raise ValueError(f"pack_scenes: {sc.name} has another gravity, dimension or dt than {s0.name}")
    if sum(len(sc.materials) for sc in scenes_) > 4096:
        raise ValueError("pack_scenes: more than 4096 materials")
    h = s0.cellsize
    boxes = []
    for sc in scenes_:
        nx, ny, nz = sc.dims()
        boxes.append((nx - 1 + 2 * margin, ny - 1 + 2 * margin, max(nz - 1, 0)))
    order = sorted(range(len(scenes_)), key=lambda i: (-boxes[i][0], i))
    area = sum(boxes[i][0] * boxes[i][1] for i in order)
    row_len = max(boxes[order[0]][0], int(math.ceil(math.sqrt(area))))
    origins = [None] * len(scenes_)
    x = y = depth = width = 0
    for i in order:
        b = boxes[i]
        if x + b[0] > row_len:
            y, x, depth = y + depth, 0, 0
        origins[i] = (x, y, 0)
        x += b[0]
        depth = max(depth, b[1])
        width = max(width, x)
    dims = (width, y + depth, max(b[2] for b in boxes))
    L = [dims[0] * h, dims[1] * h, dims[2] * h if s0.is3D else 0.0]
    nx_b, ny_b = dims[0] + 1, dims[1] + 1
    fields = {f: [] for f in ("pos", "mat", "obj", "vel", "stress", "pbc_type", "pbc_val", "hold", "temp", "flaw")}
    materials, insts, inst_of = [], [], []
    first = 0
    node_bc = []
    for i, sc in enumerate(scenes_):
        ox, oy, oz = origins[i][0] + margin, origins[i][1] + margin, 0
        shift = (ox * h, oy * h, 0.0)
        fields["pos"].append(sc.pos + np.array(shift))
        fields["mat"].append(sc.mat + len(materials))
        fields["obj"].append(sc.obj)
        for f in ("vel", "stress", "pbc_type", "pbc_val", "hold", "temp"):
            fields[f].append(getattr(sc, f))
        fields["flaw"].append(sc.flaw if sc.flaw is not None else np.ones(sc.n))
        insts.append(PackedInstance(i, sc.name, boxes[i], origins[i], shift, first, sc.n, len(materials),
                                    len(sc.materials)))
        inst_of.append(np.full(sc.n, i, np.int32))
        if sc.node_bc_type is not None and np.any(sc.node_bc_type):
            snx, sny, _ = sc.dims()
            idx = np.nonzero(sc.node_bc_type)[0]
            ii, jj, kk = idx % snx, (idx // snx) % sny, idx // (snx * sny)
            node_bc.append(((ii + ox) + (jj + oy) * nx_b + (kk + oz) * nx_b * ny_b, sc.node_bc_type[idx],
                            sc.node_bc_val[idx]))
        materials += list(sc.materials)
        first += sc.n
    pk = Scene("packed_" + "+".join(sc.name for sc in scenes_)[:200], L, h, s0.psep,
               np.concatenate(fields["pos"]), np.concatenate(fields["mat"]).astype(np.int32),
               np.concatenate(fields["obj"]).astype(np.int32), materials)
    pk.gravity, pk.damping, pk.mu, pk.CFL = list(s0.gravity), s0.damping, s0.mu, s0.CFL
    pk.fixed_grid_bcs, pk.dt = s0.fixed_grid_bcs, s0.dt
    pk.tmax = max(sc.tmax for sc in scenes_)
    for f in ("vel", "stress", "pbc_type", "pbc_val", "hold", "temp", "flaw"):
        setattr(pk, f, np.concatenate(fields[f]))
    pk.inst = np.concatenate(inst_of)
    pk.instances = insts
    pk.sources = list(scenes_)
    pk = _finish(pk, None)
    for nd, t, v in node_bc:
        pk.node_bc_type[nd] = t
        pk.node_bc_val[nd] = v
    return pk


def unpack_instance(packed: Scene, index: int) -> Scene:
    """Problem ``index`` of a :func:`pack_scenes` batch alone on its own domain, with the
    batch's dt: the scene it was packed from, in the same particle order."""
    sc = dataclasses.replace(packed.sources[index])
    if packed.dt is None:
        # the batch's dt: the Solver formula over every material row (Solver.cpp:15-32,
        # maxK seeded with 1 and the smallest density with 1e15)
        maxK = max([1.0] + [m["bulkMod"] for m in packed.materials])
        rho = min([1e15] + [m["density"] for m in packed.materials])
        sc.dt = packed.CFL * (packed.cellsize / math.sqrt(maxK / rho))
    else:
        sc.dt = packed.dt
    return sc
