"""The ``graphyt`` Python surface, GPU-backed.

Mirrors the classes the reference's SWIG module exports (graphyt.i:1-13): ``Nodes``
(Nodes.i:8-22), ``MaterialPoints`` (MaterialPoints.i:8-65), ``MaterialModels``
(MaterialModels.i:7-30), ``Parameters`` (Parameters.i:7-14), ``Solver`` (Solver.i:10-18)
and ``BCTypes`` (BoundaryConditions.hpp:6-77).  Scripts written against the reference run
unchanged up to the step call: ``Solver.iterate_GPU(t, step, params)`` advances the state
on the GPU through ``libgraphyt_gpu.so``.

Differences from the reference surface, by design:

* Particle getters return arrays indexed by insertion order (the i-th particle added).  The
  reference hands out raw pointers into arrays that its sort permutes every tenth step
  (Extrapolation.cpp:468-491), so its indices refer to a moving order.
* ``getStressXX(p)`` .. ``getStressZX(p)`` read ``stress[6p + k]``; the reference reads
  ``stress[3p + k]`` (MaterialPoints.cpp:247-252).  ``getStressArr`` is unaffected.
* ``iterate_CPU`` is the reference's own CPU step; it is not part of this package.
* Vectorised setters (``setVelocities``, ``setBCs``, ...) accept many particles at once,
  which a 12 M-particle script needs; the per-particle setters remain.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L

_BC_NAMES = [
    "none", "grid_vx", "grid_vy", "grid_vz", "grid_temp", "grid_tflux_x", "grid_tflux_y", "grid_tflux_z",
    "grid_fx", "grid_fy", "grid_fz", "grid_vx_vy", "grid_vx_vz", "grid_vy_vz", "grid_fx_fy", "grid_fy_fz",
    "grid_fx_fz", "grid_fx_fy_fz", "grid_vx_vy_vz", "grid_vx_temp", "grid_vy_temp", "grid_vz_temp",
    "grid_fx_temp", "grid_fy_temp", "grid_fz_temp", "grid_vx_vy_temp", "grid_vx_vz_temp", "grid_vy_vz_temp",
    "grid_fx_fy_temp", "grid_fy_fz_temp", "grid_fx_fz_temp", "grid_fx_fy_fz_temp", "grid_vx_vy_vz_temp",
    "mp_vx", "mp_vy", "mp_vz", "mp_temp", "mp_fx", "mp_fy", "mp_fz", "mp_vx_vy", "mp_vx_vz", "mp_vy_vz",
    "mp_fx_fy", "mp_fy_fz", "mp_fx_fz", "mp_fx_fy_fz", "mp_vx_vy_vz", "mp_vx_temp", "mp_vy_temp",
    "mp_vz_temp", "mp_fx_temp", "mp_fy_temp", "mp_fz_temp", "mp_vx_vy_temp", "mp_vx_vz_temp",
    "mp_vy_vz_temp", "mp_fx_fy_temp", "mp_fy_fz_temp", "mp_fx_fz_temp", "mp_fx_fy_fz_temp",
    "mp_vx_vy_vz_temp", "mp_stress", "mp_stress_xx_yy", "mpstrain", "mp_vxsin", "mp_vysin", "mp_syysin",
]


class BCTypes:
    """BCTypes::function (BoundaryConditions.hpp:6-77): names map to their enum values."""


for _i, _n in enumerate(_BC_NAMES):
    setattr(BCTypes, _n, _i)


class Nodes:
    """Uniform background grid, Nodes(L, cellsize) (Nodes.cpp:8-141)."""

    def __init__(self, L: Sequence[float], cellsize: float):
        self.L = [float(x) for x in L]
        self.cellsize = float(cellsize)
        h = self.cellsize
        self.Nx = int(1 + self.L[0] / h)
        self.Ny = int(1 + self.L[1] / h)
        self.Nz = int(1 + self.L[2] / h)
        self.numNodes = int(round((1 + self.L[0] / h) * (1 + self.L[1] / h) * (1 + self.L[2] / h)))
        self.numCells = int((self.L[0] / h) * (self.L[1] / h) * (self.L[2] / h))
        self.t = 0.0
        self._bc_type = np.zeros(self.numNodes, np.int32)
        self._bc_val = np.zeros((self.numNodes, 4))
        self._solver: Optional["Solver"] = None

    def setBC(self, nIdx: int, type: int, val: Sequence[float]):
        self._bc_type[nIdx] = int(type)
        v = list(val)[:4]
        self._bc_val[nIdx, : len(v)] = v

    def setBCs(self, idx, type, val):
        """Vectorised setBC: idx (k,), type (k,) or scalar, val (k, <=4)."""
        idx = np.asarray(idx, np.int64)
        self._bc_type[idx] = type
        val = np.atleast_2d(np.asarray(val, np.float64))
        self._bc_val[idx, : val.shape[1]] = val

    def _pos(self, n: int):
        i = n % self.Nx
        j = (n // self.Nx) % self.Ny
        k = n // (self.Nx * self.Ny)
        return i * self.cellsize, j * self.cellsize, k * self.cellsize

    def getPosX(self, n):
        return self._pos(n)[0]

    def getPosY(self, n):
        return self._pos(n)[1]

    def getPosZ(self, n):
        return self._pos(n)[2]

    def getPosArr(self) -> np.ndarray:
        k, j, i = np.meshgrid(np.arange(self.Nz), np.arange(self.Ny), np.arange(self.Nx), indexing="ij")
        return np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64).ravel() * self.cellsize

    def _node_field(self, name: str, width: int) -> np.ndarray:
        if self._solver is None:
            return np.zeros(self.numNodes * width)
        return self._solver._get_nodes(name, width).ravel()

    def getMassArr(self):
        return self._node_field("mass", 1)

    def getVelArr(self):
        return self._node_field("vel", 3)

    def getForceArr(self):
        return self._node_field("force", 3)

    def Serialise(self, step: int, filename: str):
        """CSV of node positions, as Nodes::Serialise (Nodes.cpp:165-177)."""
        pos = self.getPosArr().reshape(-1, 3)
        with open(f"output/{filename}_nds_{step}.csv", "w") as f:
            f.write("Pos_x,Pos_y,Pos_z\n")
            for p in pos:
                f.write("%f,%f,%f\n" % tuple(p))


class MaterialPoints:
    """Particle set, MaterialPoints(nodes) (MaterialPoints.cpp:10-17)."""

    def __init__(self, nodes: Nodes):
        self.nodes = nodes
        self.psep = 0.0
        self.t = 0.0
        self._pos: List[np.ndarray] = []
        self._n = 0
        self._mat = None
        self._obj = None
        self._vel = {}
        self._stress = {}
        self._damage = {}
        self._flaw = None
        self._temp = {}
        self._hold = set()
        self._bc = {}
        self._solver: Optional["Solver"] = None

    # ---- construction -------------------------------------------------------------------
    @property
    def numParticles(self) -> int:
        return self._n

    def add(self, i: int, x: float, y: float, z: float):
        self._pos.append(np.array([[x, y, z]], np.float64))
        self._n += 1

    def addPyckGeom(self, pos, numParticles: int):
        p = np.asarray(pos, np.float64).reshape(-1)[: 3 * int(numParticles)].reshape(-1, 3)
        self._pos.append(p.copy())
        self._n += len(p)

    def addPyckIntField(self, field):
        """field has .name ('material' or 'objectID') and .data (ints), like pyck's IntField."""
        data = np.asarray(field.data, np.int32)[: self._n]
        if field.name == "material":
            self._mat = data.copy()
        elif field.name == "objectID":
            self._obj = data.copy()

    def _positions(self) -> np.ndarray:
        if not self._pos:
            return np.zeros((0, 3))
        if len(self._pos) > 1:
            self._pos = [np.concatenate(self._pos)]
        return self._pos[0]

    def _ids(self, which):
        arr = self._mat if which == "mat" else self._obj
        if arr is None:
            arr = np.zeros(self._n, np.int32)
            if which == "mat":
                self._mat = arr
            else:
                self._obj = arr
        return arr

    def setMaterialID(self, p, materialID):
        self._ids("mat")[p] = materialID

    def setObjectID(self, p, objid):
        self._ids("obj")[p] = objid

    def setVel(self, p, vx, vy, vz):
        self._vel[int(p)] = (vx, vy, vz)

    def setVelocities(self, idx, vel):
        for p, v in zip(np.asarray(idx).tolist(), np.asarray(vel, np.float64).reshape(-1, 3).tolist()):
            self._vel[int(p)] = tuple(v)

    def setStress(self, p, sxx, syy, szz, sxy, syz, sxz):
        self._stress[int(p)] = (sxx, syy, szz, sxy, syz, sxz)

    def setDamage(self, p, D):
        self._damage[int(p)] = float(D)

    def setFlawScales(self, w):
        """Per-particle scale of the Grady-Kipp activation strain, e_min = w (V k)^(-1/m), one
        value per particle in insertion order (1 everywhere is the reference's deterministic
        e_min, DamageModels.cpp:102-103; scenes.weibull_flaws draws Weibull scales).  No
        reference counterpart."""
        self._flaw = np.ascontiguousarray(w, np.float64).reshape(-1)

    def setTemp(self, p, T):
        """MaterialPoints::setTemp (MaterialPoints.cpp:319-322); also between steps."""
        self.setTemps([p], [T])

    def setTemps(self, idx, T):
        """setTemp for many particles at once."""
        idx = np.asarray(idx, np.int64).ravel()
        T = np.broadcast_to(np.asarray(T, np.float64).ravel(), idx.shape)
        if self._solver is None:
            for p, t in zip(idx.tolist(), T.tolist()):
                self._temp[int(p)] = float(t)
        else:
            self._solver._set_temps(idx, T)

    def holdParticle(self, p):
        self._hold.add(int(p))

    def setBC(self, p, type, val):
        """MaterialPoints::setBC (MaterialPoints.cpp:88-93): writes the type and only the values
        given; the others keep what an earlier call set (zero at first, :210-217)."""
        v = list(self._bc.get(int(p), (0, [0.0] * 4))[1])
        given = [float(x) for x in list(val)[:4]]
        v[: len(given)] = given
        self._bc[int(p)] = (int(type), v)

    def setBCs(self, idx, type, val):
        """setBC for many particles at once: idx (k,), type (k,) or scalar, val (k, <=4) or (<=4,)."""
        val = np.atleast_2d(np.asarray(val, np.float64))
        types = np.broadcast_to(np.asarray(type, np.int32), (len(idx),))
        for q, p in enumerate(np.asarray(idx).tolist()):
            self.setBC(p, types[q], val[q if len(val) > 1 else 0].tolist())

    # ---- getters (MaterialPoints.cpp:238-273) --------------------------------------------
    def _field(self, name):
        if self._solver is None:
            raise RuntimeError("particle state lives on the GPU once a Solver exists; create the Solver first")
        return self._solver._get_particles(name)

    def getPosArr(self):
        return self._field("pos").ravel()

    def getDispArr(self):
        return self._field("disp").ravel()

    def getVelArr(self):
        return self._field("vel").ravel()

    def getStressArr(self):
        return self._field("stress").ravel()

    def getStrainArr(self):
        return self._field("strain").ravel()

    def getPlasticStrainArr(self):
        return self._field("pstrain").ravel()

    def getTemperatureArr(self):
        return self._field("temp").ravel()

    def getAccPlasticStrainArr(self):
        return self._field("eqps").ravel()

    def getDamageArr(self):
        return self._field("damage").ravel()

    def getSMaxArr(self):
        return self._field("smax").ravel()

    def getMassArr(self):
        return self._field("mass").ravel()

    def getDensityArr(self):
        return self._field("density").ravel()

    def getVolumeArr(self):
        return self._field("volume").ravel()

    def getNormalsArr(self):
        return self._field("normals").ravel()

    def getMatArr(self):
        return self._solver._get_particles_int("material") if self._solver else self._ids("mat").copy()

    def getObjectIDArr(self):
        return self._solver._get_particles_int("object") if self._solver else self._ids("obj").copy()

    def getCellIDArr(self):
        return self._solver._get_particles_int("cellid")

    def getPosX(self, p):
        return float(self._field("pos")[p, 0])

    def getPosY(self, p):
        return float(self._field("pos")[p, 1])

    def getPosZ(self, p):
        return float(self._field("pos")[p, 2])

    def getDispX(self, p):
        return float(self._field("disp")[p, 0])

    def getDispY(self, p):
        return float(self._field("disp")[p, 1])

    def getDispZ(self, p):
        return float(self._field("disp")[p, 2])

    def getVelX(self, p):
        return float(self._field("vel")[p, 0])

    def getVelY(self, p):
        return float(self._field("vel")[p, 1])

    def getVelZ(self, p):
        return float(self._field("vel")[p, 2])

    def getStressXX(self, p):
        return float(self._field("stress")[p, 0])

    def getStressYY(self, p):
        return float(self._field("stress")[p, 1])

    def getStressZZ(self, p):
        return float(self._field("stress")[p, 2])

    def getStressXY(self, p):
        return float(self._field("stress")[p, 3])

    def getStressYZ(self, p):
        return float(self._field("stress")[p, 4])

    def getStressZX(self, p):
        return float(self._field("stress")[p, 5])

    def getObjID(self, p):
        return int(self.getObjectIDArr()[p])

    def getMatID(self, p):
        return int(self.getMatArr()[p])

    def getCellID(self, p):
        return int(self.getCellIDArr()[p])

    def Serialise(self, step: int, filename: str):
        """CSV like MaterialPoints::Serialise (MaterialPoints.cpp:341-364)."""
        x = self._field("pos")
        v = self._field("vel")
        s = self._field("stress")
        rho = self._field("density").ravel()
        T = self._field("temp").ravel()
        vm = np.sqrt(s[:, 0] ** 2 + s[:, 1] ** 2 + s[:, 2] ** 2 + (2 * s[:, 3]) ** 2 + (2 * s[:, 4]) ** 2 + (2 * s[:, 5]) ** 2)
        P = 0.33 * (s[:, 0] + s[:, 1] + s[:, 2])
        with open(f"output/{filename}_mpts_{step}.csv", "w") as f:
            f.write("x,y,z,vm,P,T,vx,vy,vz,rho\n")
            for i in range(len(x)):
                f.write("%f,%f,%f,%f,%f,%f,%f,%f,%f,%f\n" % (x[i, 0], x[i, 1], x[i, 2], vm[i], P[i], T[i],
                                                           v[i, 0], v[i, 1], v[i, 2], rho[i]))


class MaterialModels:
    """Material properties with the reference's defaults (MaterialModels.cpp:4-26)."""

    def __init__(self):
        self.bulkMod = 1e7
        self.shearMod = 5000.0
        self.density = 1000.0
        self.isRigid = False
        self.viscosity = 1.0
        self.thermalConductivity = 391.0
        self.specificHeatCapacity = 385.2
        self.yieldStress = 1e7
        self.phi = 40.0
        self.psi = 10.0
        self.cohesion = 100000.0
        self.criticalStrain = 0.01
        self.isDamage = False
        self.damageModel = 1
        self.Cg = 586.52
        self.damageM = 9.0
        self.damageK = 5.39e36
        self.turbStress = 1e10
        self.model = 1

    def setBulkMod(self, v): self.bulkMod = float(v)
    def setShearMod(self, v): self.shearMod = float(v)
    def setDensity(self, v): self.density = float(v)
    def setIsRigid(self, v): self.isRigid = bool(v)
    def setViscosity(self, v): self.viscosity = float(v)
    def setThermalConductivity(self, v): self.thermalConductivity = float(v)
    def setSpecificHeatCapacity(self, v): self.specificHeatCapacity = float(v)
    def setYieldStress(self, v): self.yieldStress = float(v)
    def setCohesion(self, v): self.cohesion = float(v)
    def setCriticalStrain(self, v): self.criticalStrain = float(v)
    def setFrictionAngle(self, v): self.phi = float(v)
    def setDilatancyAngle(self, v): self.psi = float(v)
    def setIsDamage(self, v): self.isDamage = bool(v)
    def setDamageModel(self, v): self.damageModel = int(v)
    def setCrackSpeed(self, v): self.Cg = float(v)
    def setDamageM(self, v): self.damageM = float(v)
    def setDamageK(self, v): self.damageK = float(v)
    def setTurbulentStress(self, v): self.turbStress = float(v)
    def setModel(self, v): self.model = int(v)

    def _ctype(self) -> L.Material:
        m = L.Material()
        for f in L.MAT_DOUBLE_FIELDS:
            setattr(m, f, float(getattr(self, f)))
        m.isRigid = int(bool(self.isRigid))
        m.isDamage = int(bool(self.isDamage))
        m.damageModel = int(self.damageModel)
        m.model = int(self.model)
        return m


class Parameters:
    """Parameters(tmax, is3D) (Parameters.cpp:8-15).  The reference leaves gravity
    uninitialised until setGravity; here it starts at zero."""

    def __init__(self, tmax: float, is3D: bool):
        self.tmax = float(tmax)
        self.is3D = bool(is3D)
        self.CFL = 0.1
        self.mu = 0.0
        self.velocityDampingCoef = 0.0
        self.gravity = [0.0, 0.0, 0.0]
        self.dt = 0.0
        self.fixed_grid_bcs = 0

    def setGravity(self, gx, gy, gz):
        self.gravity = [float(gx), float(gy), float(gz)]

    def setDampingCoef(self, c):
        self.velocityDampingCoef = float(c)

    def setCFL(self, cfl):
        self.CFL = float(cfl)

    def setFriction(self, mu):
        self.mu = float(mu)

    def setFixedGridBCs(self, on: bool):
        """Give grid_vz, grid_vx_vz, grid_vy_vz and grid_vx_vy_vz a body (empty in the
        reference, Grid.cpp:872-873, 1032-1052)."""
        self.fixed_grid_bcs = 1 if on else 0

    def _ctype(self) -> L.Params:
        p = L.Params()
        for k in range(3):
            p.gravity[k] = self.gravity[k]
        p.damping = self.velocityDampingCoef
        p.mu = self.mu
        p.CFL = self.CFL
        p.tmax = self.tmax
        p.is3D = 1 if self.is3D else 0
        p.fixed_grid_bcs = int(self.fixed_grid_bcs)
        return p


class Solver:
    """Solver(nds, mpts, params, materials) (Solver.cpp:7-37) on the GPU."""

    def __init__(self, nds: Nodes, mpts: MaterialPoints, mpmParameters: Parameters, materials,
                 device: int = -1, options: Optional[dict] = None):
        self.lib = L.load()
        self.nds, self.mpts, self.params = nds, mpts, mpmParameters
        self.materials = list(materials)
        g = L.GridDesc()
        for k in range(3):
            g.L[k] = nds.L[k]
        g.cellsize = nds.cellsize
        if not mpts.psep > 0:
            raise ValueError("MaterialPoints.psep must be set before the Solver is built")
        g.psep = mpts.psep
        h = C.c_void_p()
        rc = self.lib.gy_create(C.byref(g), int(device), C.byref(h))
        if rc != 0:
            raise L.GraphytGPUError(rc, "gy_create: grid rejected (Nx*Ny*Nz must equal numNodes, psep <= cellsize)")
        self.h = h
        try:
            self._upload(options or {})
        except Exception:
            self.close()
            raise
        self.startTimeLoop = 0.0
        nds._solver = self
        mpts._solver = self

    def _upload(self, options: dict):
        lib, h, mp = self.lib, self.h, self.mpts
        pos = np.ascontiguousarray(mp._positions(), np.float64)
        n = len(pos)
        mat = np.ascontiguousarray(mp._ids("mat"), np.int32)
        obj = np.ascontiguousarray(mp._ids("obj"), np.int32)
        L.check(lib.gy_add_particles(h, n, L.dptr(pos), L.iptr(mat), L.iptr(obj)), h, "gy_add_particles")
        if mp._vel:
            idx = np.fromiter(mp._vel.keys(), np.int64)
            v = np.ascontiguousarray(np.array(list(mp._vel.values()), np.float64).reshape(-1, 3))
            L.check(lib.gy_set_particle_vel(h, len(idx), L.i64ptr(idx), L.dptr(v)), h, "setVel")
        if mp._stress:
            idx = np.fromiter(mp._stress.keys(), np.int64)
            s = np.ascontiguousarray(np.array(list(mp._stress.values()), np.float64).reshape(-1, 6))
            L.check(lib.gy_set_particle_stress(h, len(idx), L.i64ptr(idx), L.dptr(s)), h, "setStress")
        if mp._damage:
            idx = np.fromiter(mp._damage.keys(), np.int64)
            d = np.ascontiguousarray(np.array(list(mp._damage.values()), np.float64))
            L.check(lib.gy_set_particle_damage(h, len(idx), L.i64ptr(idx), L.dptr(d)), h, "setDamage")
        if mp._flaw is not None:
            w = mp._flaw
            if len(w) != mp._n:
                raise ValueError("setFlawScales: one scale per particle")
            idx = np.arange(len(w), dtype=np.int64)
            L.check(lib.gy_set_particle_flaw(h, len(idx), L.i64ptr(idx), L.dptr(w)), h, "setFlawScales")
        if mp._temp:
            idx = np.fromiter(mp._temp.keys(), np.int64)
            t = np.ascontiguousarray(np.fromiter(mp._temp.values(), np.float64))
            L.check(lib.gy_set_particle_temp(h, len(idx), L.i64ptr(idx), L.dptr(t)), h, "setTemp")
        if mp._hold:
            idx = np.array(sorted(mp._hold), np.int64)
            L.check(lib.gy_hold_particles(h, len(idx), L.i64ptr(idx)), h, "holdParticle")
        if mp._bc:
            idx = np.fromiter(mp._bc.keys(), np.int64)
            t = np.array([b[0] for b in mp._bc.values()], np.int32)
            v = np.ascontiguousarray(np.array([b[1] for b in mp._bc.values()], np.float64).reshape(-1, 4))
            L.check(lib.gy_set_particle_bc(h, len(idx), L.i64ptr(idx), L.iptr(t), L.dptr(v)), h, "setBC")
        nz = np.nonzero(self.nds._bc_type)[0].astype(np.int64)
        if len(nz):
            t = np.ascontiguousarray(self.nds._bc_type[nz], np.int32)
            v = np.ascontiguousarray(self.nds._bc_val[nz], np.float64)
            L.check(lib.gy_set_node_bc(h, len(nz), L.i64ptr(nz), L.iptr(t), L.dptr(v)), h, "Nodes.setBC")
        self.set_options(**options)
        mats = (L.Material * len(self.materials))(*[m._ctype() for m in self.materials])
        prm = self.params._ctype()
        L.check(lib.gy_initialize(h, mats, len(self.materials), C.byref(prm)), h, "gy_initialize")

    # ---- reference surface ----------------------------------------------------------------
    @property
    def dt(self) -> float:
        d = C.c_double()
        L.check(self.lib.gy_get_dt(self.h, C.byref(d)), self.h)
        return d.value

    @dt.setter
    def dt(self, value: float):
        self.setDt(value)

    @property
    def tmax(self) -> float:
        return self.params.tmax

    def setDt(self, dt: float):
        L.check(self.lib.gy_set_dt(self.h, float(dt)), self.h, "setDt")

    def iterate_GPU(self, t: float, step: int, mpmParameters: Optional[Parameters] = None):
        """One explicit step on the GPU (the GPU counterpart of iterate_CPU, Solver.cpp:86-292)."""
        if mpmParameters is not None:
            prm = mpmParameters._ctype()
            L.check(self.lib.gy_set_params(self.h, C.byref(prm)), self.h, "parameters")
        L.check(self.lib.gy_step(self.h, float(t), int(step)), self.h, "iterate_GPU")
        self.mpts.t = t
        self.nds.t = t

    def iterate_GPU_steps(self, nsteps: int, mpmParameters: Optional[Parameters] = None, step0: int = 0,
                          t0: float = 0.0, use_graph: bool = True):
        """nsteps consecutive steps from step0 (iterate_CPU_steps, Solver.cpp:75-84)."""
        if mpmParameters is not None:
            prm = mpmParameters._ctype()
            L.check(self.lib.gy_set_params(self.h, C.byref(prm)), self.h, "parameters")
        L.check(self.lib.gy_steps(self.h, float(t0), int(step0), int(nsteps), 1 if use_graph else 0), self.h,
                "iterate_GPU_steps")

    def iterate_CPU(self, *args, **kwargs):
        raise NotImplementedError("iterate_CPU is the reference's CPU step; this package runs the step on the "
                                  "GPU: call iterate_GPU(t, step, params)")

    def iterate_CPU_steps(self, *args, **kwargs):
        raise NotImplementedError("use iterate_GPU_steps")

    def Synchronise(self):
        L.check(self.lib.gy_sync(self.h), self.h, "sync")

    # ---- extras ---------------------------------------------------------------------------
    def set_options(self, **kw):
        o = L.Options()
        L.check(self.lib.gy_get_options(self.h, C.byref(o)), self.h)
        for k, v in kw.items():
            if not hasattr(o, k):
                raise KeyError(k)
            setattr(o, k, int(v))
        L.check(self.lib.gy_set_options(self.h, C.byref(o)), self.h, "options")

    def _single_body(self) -> bool:
        """Whether the step runs the single-body kernels: one object, no rigid material, no
        tracked contact normals (the library's rule at gy_initialize)."""
        o = L.Options()
        L.check(self.lib.gy_get_options(self.h, C.byref(o)), self.h)
        objs = self.mpts._obj
        n_obj = len(np.unique(objs)) if objs is not None and len(objs) else 1
        mats = self.mpts._mat
        used = np.unique(mats) if mats is not None and len(mats) else np.array([0])
        rigid = any(bool(getattr(self.materials[int(m)], "isRigid", 0)) for m in used if int(m) < len(self.materials))
        return n_obj <= 1 and not rigid and not o.track_normals

    def autotune(self, step0: int = 0, steps: int = 6,
                 candidates=((1, 0), (2, 0), (4, 0), (1, 1)), lanes=(3, 9)) -> dict:
        """Choose the fastest step configuration for this problem and keep it.

        Two stages: the sort cadence and kind (``candidates``: (sort_every, full_sort) pairs),
        then, with those fixed, the P2G lane mapping (``lanes``: 3 z-plane lanes per run of
        equal cell, ten runs per warp, or 9 x-column lanes, three runs per warp -- how many
        particles a warp sums at once; on multi-body problems, whether the one-object segments
        take the 3-lane kernel or all take the body-slot kernel).  Each candidate runs a few untimed steps (its
        CUDA graphs are captured there), then ``steps`` steps timed with CUDA events.  These
        are real steps of the run, from step ``step0`` on, since the knobs change speed and
        never results beyond summation order; the returned ``next_step`` is where the caller
        continues.  The cell block (4^3 cells and its 6^3-node shared-memory tile) is fixed by
        the kernels' key encoding; multi-body problems that track normals skip the lane stage
        (every segment takes the body-slot kernel there)."""
        ms = C.c_float()
        dt = self.dt
        step = int(step0)

        def timed(**opts):
            nonlocal step
            self.set_options(**opts)
            warm = max(2, 2 * int(opts.get("sort_every", 1)))
            L.check(self.lib.gy_steps(self.h, step * dt, step, warm, 1), self.h, "autotune")
            step += warm
            L.check(self.lib.gy_time_steps(self.h, step * dt, step, int(steps), C.byref(ms)), self.h, "autotune")
            step += int(steps)
            return ms.value / max(int(steps), 1)

        times = {}
        for sort_every, full_sort in candidates:
            times[(int(sort_every), int(full_sort))] = timed(sort_every=int(sort_every), full_sort=int(full_sort))
        best = min(times, key=times.get)
        lane_times = {}
        o = L.Options()
        L.check(self.lib.gy_get_options(self.h, C.byref(o)), self.h)
        best_lanes = int(o.p2g_lanes)
        if self._single_body() or not o.track_normals:  # tracked normals: the body-slot kernel only
            for ln in lanes:
                lane_times[int(ln)] = timed(sort_every=best[0], full_sort=best[1], p2g_lanes=int(ln))
            best_lanes = min(lane_times, key=lane_times.get)
        self.set_options(sort_every=best[0], full_sort=best[1], p2g_lanes=best_lanes)
        return dict(sort_every=best[0], full_sort=best[1], p2g_lanes=best_lanes, ms_per_step=times,
                    lanes_ms_per_step=lane_times, next_step=step)

    # ---- learned Drucker-Prager surrogate (no reference counterpart) ------------------------
    def dp_log_begin(self, cap: int, every: int = 1):
        """Record (strain increment, state) -> (return correction, plastic strain increment)
        pairs of yielding Drucker-Prager particles from the exact return mapping of the coming
        steps, up to cap records, one particle in `every`."""
        L.check(self.lib.gy_dp_log_begin(self.h, int(cap), int(every)), self.h, "dp_log_begin")

    def dp_log_end(self):
        L.check(self.lib.gy_dp_log_end(self.h), self.h, "dp_log_end")

    def dp_log_count(self) -> int:
        c = C.c_int64()
        L.check(self.lib.gy_dp_log_count(self.h, C.byref(c)), self.h, "dp_log_count")
        return int(c.value)

    def dp_log_read(self):
        """The logged records as (inputs [m][16], targets [m][7]) float32 arrays."""
        m = self.dp_log_count()
        x = np.empty((m, 16), np.float32)
        y = np.empty((m, 7), np.float32)
        if m:
            L.check(self.lib.gy_dp_log_read(self.h, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), m),
                    self.h, "dp_log_read")
        return x, y

    def train_surrogate(self, steps: int = 20000, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
        """Train the surrogate MLP on the logged records on the GPU; returns the final loss."""
        loss = C.c_float()
        L.check(self.lib.gy_dp_surrogate_train(self.h, int(steps), int(batch), C.c_float(lr), int(seed),
                                               C.byref(loss)), self.h, "train_surrogate")
        return float(loss.value)

    def set_surrogate(self, on: bool = True, params=None, tol: float = 1e-4):
        """Switch the surrogate return mapping on or off; params (gy_mlp_param_count floats)
        replace the trained parameters when given."""
        p = None
        if params is not None:
            params = np.ascontiguousarray(params, np.float32)
            p = params.ctypes.data_as(C.c_void_p)
        L.check(self.lib.gy_set_dp_surrogate(self.h, p, 1 if on else 0, C.c_float(tol)), self.h, "set_surrogate")

    def surrogate_params(self) -> np.ndarray:
        out = np.empty(int(self.lib.gy_mlp_param_count()), np.float32)
        L.check(self.lib.gy_get_dp_surrogate(self.h, out.ctypes.data_as(C.c_void_p)), self.h, "surrogate_params")
        return out

    def surrogate_counts(self) -> dict:
        k, f = C.c_int64(), C.c_int64()
        L.check(self.lib.gy_dp_surrogate_counts(self.h, C.byref(k), C.byref(f)), self.h, "surrogate_counts")
        return dict(kept=int(k.value), fallback=int(f.value))

    def _set_temps(self, idx, T):
        idx = np.ascontiguousarray(idx, np.int64)
        T = np.ascontiguousarray(T, np.float64)
        L.check(self.lib.gy_set_particle_temp(self.h, len(idx), L.i64ptr(idx), L.dptr(T)), self.h, "setTemp")

    def save(self, path: str):
        """Write a binary snapshot of the device state (checkpoint); resume with load()."""
        nbytes = C.c_int64()
        L.check(self.lib.gy_state_size(self.h, C.byref(nbytes)), self.h, "state size")
        buf = np.empty(nbytes.value, np.uint8)
        L.check(self.lib.gy_state_save(self.h, buf.ctypes.data_as(C.c_void_p), buf.size), self.h, "save")
        with open(path, "wb") as f:
            f.write(buf.tobytes())

    def load(self, path: str):
        """Restore a snapshot written by save() into a Solver built from the same model."""
        buf = np.fromfile(path, np.uint8)
        L.check(self.lib.gy_state_load(self.h, buf.ctypes.data_as(C.c_void_p), buf.size), self.h, "load")

    def stats(self) -> dict:
        s = L.Stats()
        L.check(self.lib.gy_get_stats(self.h, C.byref(s)), self.h, "stats")
        return dict(mass=s.mass, momentum=list(s.momentum), kinetic=s.kinetic, strain_energy=s.strain_energy,
                    active_nodes=s.active_nodes, steps=s.steps, status_flags=s.status_flags)

    def stream(self) -> int:
        return self.lib.gy_stream(self.h) or 0

    def _get_particles(self, name: str) -> np.ndarray:
        n = C.c_int64()
        L.check(self.lib.gy_num_particles(self.h, C.byref(n)), self.h)
        w = L.P_WIDTH[name]
        out = np.empty((n.value, w), np.float64)
        L.check(self.lib.gy_get_particles(self.h, L.P_FIELDS[name], L.dptr(out), out.size), self.h, name)
        return out if w > 1 else out[:, 0]

    def _get_particles_int(self, name: str) -> np.ndarray:
        n = C.c_int64()
        L.check(self.lib.gy_num_particles(self.h, C.byref(n)), self.h)
        out = np.empty(n.value, np.int32)
        L.check(self.lib.gy_get_particles_int(self.h, L.PI_FIELDS[name], L.iptr(out), out.size), self.h, name)
        return out

    def _get_nodes(self, name: str, width: int) -> np.ndarray:
        out = np.empty((self.nds.numNodes, width), np.float64)
        L.check(self.lib.gy_get_nodes(self.h, L.N_FIELDS[name], L.dptr(out), out.size), self.h, name)
        return out if width > 1 else out[:, 0]

    def close(self):
        if getattr(self, "h", None):
            self.lib.gy_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _IntField:
    def __init__(self, name, data):
        self.name, self.data = name, data


def from_scene(scene, device: int = -1, options: Optional[dict] = None) -> Solver:
    """Build Nodes / MaterialPoints / MaterialModels / Parameters / Solver from a
    :class:`graphyt_gb300.scenes.Scene` through the reference-shaped surface."""
    nodes = Nodes(scene.L, scene.cellsize)
    mp = MaterialPoints(nodes)
    mp.psep = scene.psep
    mp.addPyckGeom(scene.pos, scene.n)
    mp.addPyckIntField(_IntField("material", scene.mat))
    mp.addPyckIntField(_IntField("objectID", scene.obj))
    nzv = np.nonzero(np.any(scene.vel != 0, axis=1))[0]
    mp._vel = {int(p): tuple(scene.vel[p]) for p in nzv}
    nzs = np.nonzero(np.any(scene.stress != 0, axis=1))[0]
    mp._stress = {int(p): tuple(scene.stress[p]) for p in nzs}
    mp._hold = set(np.nonzero(scene.hold)[0].tolist())
    temp = getattr(scene, "temp", None)
    if temp is not None:
        mp._temp = {int(p): float(temp[p]) for p in np.nonzero(temp)[0]}
    flaw = getattr(scene, "flaw", None)
    if flaw is not None and np.any(flaw != 1.0):
        mp.setFlawScales(flaw)
    nzb = np.nonzero(scene.pbc_type)[0]
    mp._bc = {int(p): (int(scene.pbc_type[p]), list(scene.pbc_val[p])) for p in nzb}
    nodes._bc_type = scene.node_bc_type.astype(np.int32).copy()
    nodes._bc_val = scene.node_bc_val.astype(np.float64).copy()
    mats = []
    for m in scene.materials:
        mm = MaterialModels()
        for k, v in m.items():
            setattr(mm, k, v)
        mats.append(mm)
    prm = Parameters(scene.tmax, scene.is3D)
    prm.setGravity(*scene.gravity)
    prm.setDampingCoef(scene.damping)
    prm.setCFL(scene.CFL)
    prm.setFriction(scene.mu)
    prm.setFixedGridBCs(bool(scene.fixed_grid_bcs))
    solver = Solver(nodes, mp, prm, mats, device=device, options=options)
    if scene.dt is not None:
        solver.setDt(scene.dt)
    return solver
