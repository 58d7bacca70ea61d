"""ctypes driver for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads one of two shared libraries built by ``oracle/Makefile``:

* ``kind="port"``: ``_build/liboracle.so``, the FP64 restatement in ``gy_oracle.c``;
* ``kind="ref"``:  ``_ref/libgyref.so``, the unmodified reference sources driven by
  ``ref_harness.cpp`` (only where the reference tree was available at build time).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
# the reference source tree, where one exists (not on machines that only run the GPU tests)
REFERENCE_DIR = os.environ.get("GRAPHYT_REFERENCE", "/root/reference")
REF_LIB = os.path.join(HERE, "_ref", "libgyref.so")

P_FIELDS = dict(pos=0, pos0=1, disp=2, vel=3, gvel=4, acc=5, strainrate=6, stress=7, strain=8,
                pstrain=9, eqps=10, damage=11, smax=12, mass=13, density=14, volume=15, normals=16,
                densityrate=17, temp=18, tempgrad=19)
P_WIDTH = dict(pos=3, pos0=3, disp=3, vel=3, gvel=3, acc=3, strainrate=6, stress=6, strain=6,
               pstrain=6, eqps=1, damage=1, smax=1, mass=1, density=1, volume=1, normals=3,
               densityrate=1, temp=1, tempgrad=3)
PI_FIELDS = dict(cell=0, mat=1, obj=2, pid=3)
N_FIELDS = dict(mass=0, mass1=1, mass2=2, mom=3, mom1=4, mom2=5, force=6, force1=7, force2=8,
                vel=9, vel1=10, vel2=11, acc1=12, acc2=13, normal1=14, normal2=15, temp=16, temprate=17)
NI_FIELDS = dict(body=0, rigid=1, cells=2, cellcount=3)

MAT_DOUBLE_FIELDS = ["bulkMod", "shearMod", "density", "viscosity", "thermalConductivity",
                     "specificHeatCapacity", "yieldStress", "cohesion", "criticalStrain", "phi",
                     "psi", "Cg", "damageM", "damageK", "turbStress"]
MAT_INT_FIELDS = ["isRigid", "isDamage", "damageModel", "model"]


class Material(C.Structure):
    _fields_ = [(f, C.c_double) for f in MAT_DOUBLE_FIELDS] + [(f, C.c_int) for f in MAT_INT_FIELDS]


class Params(C.Structure):
    _fields_ = [("gravity", C.c_double * 3), ("damping", C.c_double), ("mu", C.c_double),
                ("CFL", C.c_double), ("tmax", C.c_double), ("is3D", C.c_int),
                ("fixed_grid_bcs", C.c_int)]


def build(reference: Optional[str] = None, quiet: bool = True) -> None:
    """Compile the restatement, and the reference library when the reference tree exists."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=out)
    ref = reference or REFERENCE_DIR
    if os.path.isdir(ref):
        subprocess.run(["make", "-C", HERE, "ref", f"REFERENCE={ref}"], check=True, stdout=out)


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind == "port" else REF_LIB)


_LIBS = {}


def _lib(kind: str):
    if kind in _LIBS:
        return _LIBS[kind], ("gyo_" if kind == "port" else "gyr_")
    path = PORT_LIB if kind == "port" else REF_LIB
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library {path} is not built (make -C oracle)")
    lib = C.CDLL(path)
    pre = "gyo_" if kind == "port" else "gyr_"
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "create": (vp, [C.c_double] * 5),
        "destroy": (None, [vp]),
        "add_particles": (C.c_int, [vp, C.c_int, dp, ip, ip]),
        "set_particle_vel": (None, [vp, C.c_int, C.c_double, C.c_double, C.c_double]),
        "set_particle_stress": (None, [vp, C.c_int, dp]),
        "set_particle_damage": (None, [vp, C.c_int, C.c_double]),
        "hold_particle": (None, [vp, C.c_int]),
        "set_particle_bc": (None, [vp, C.c_int, C.c_int, dp, C.c_int]),
        "set_node_bc": (None, [vp, C.c_int, C.c_int, dp, C.c_int]),
        "set_particle_temps": (None, [vp, C.c_int, ip, dp]),
        "init_solver": (C.c_int, [vp, C.POINTER(Params), C.c_int, C.POINTER(Material)]),
        "get_dt": (C.c_double, [vp]),
        "set_dt": (None, [vp, C.c_double]),
        "set_params": (None, [vp, C.POINTER(Params)]),
        "num_particles": (C.c_int, [vp]),
        "num_nodes": (C.c_int, [vp]),
        "dims": (None, [vp, ip]),
        "get_particle_field": (C.c_int, [vp, C.c_int, dp]),
        "get_particle_ifield": (C.c_int, [vp, C.c_int, ip]),
        "get_node_field": (C.c_int, [vp, C.c_int, dp]),
        "get_node_ifield": (C.c_int, [vp, C.c_int, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, pre + name)
        f.restype = res
        f.argtypes = args
    step = getattr(lib, pre + "step")
    step.restype = C.c_int
    step.argtypes = [vp, C.c_double, C.c_int] + ([] if kind == "port" else [C.c_int])
    if kind == "port":
        lib.gyo_set_particle_flaws.restype = None
        lib.gyo_set_particle_flaws.argtypes = [vp, C.c_int, ip, dp]
        lib.gyo_gimp_shape.restype = C.c_double
        lib.gyo_gimp_shape.argtypes = [C.c_double] * 3
        lib.gyo_gimp_grad.restype = C.c_double
        lib.gyo_gimp_grad.argtypes = [C.c_double] * 4
        lib.gyo_sym_eigen.restype = C.c_int
        lib.gyo_sym_eigen.argtypes = [dp, dp, dp]
    _LIBS[kind] = lib
    return lib, pre


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def make_params(scene) -> Params:
    p = Params()
    for k in range(3):
        p.gravity[k] = float(scene.gravity[k])
    p.damping = float(scene.damping)
    p.mu = float(scene.mu)
    p.CFL = float(scene.CFL)
    p.tmax = float(scene.tmax)
    p.is3D = 1 if scene.is3D else 0
    p.fixed_grid_bcs = int(scene.fixed_grid_bcs)
    return p


def make_materials(mats):
    arr = (Material * len(mats))()
    for i, m in enumerate(mats):
        for f in MAT_DOUBLE_FIELDS:
            setattr(arr[i], f, float(m[f]))
        for f in MAT_INT_FIELDS:
            setattr(arr[i], f, int(m[f]))
    return arr


class Oracle:
    """One CPU simulation built from a :class:`graphyt_gb300.scenes.Scene`.

    ``mode`` (reference library only): 0 = the literal ``Solver::iterate_CPU``; 1 = the
    harness sequence with the (cellID, particle id) sort and optional fixed grid BCs.  The
    restatement always follows harness semantics.
    """

    def __init__(self, scene, kind: str = "port", mode: int = 1):
        self.kind, self.mode, self.scene = kind, mode, scene
        self.lib, self.pre = _lib(kind)
        L = scene.L
        self.h = self._call("create", L[0], L[1], L[2], scene.cellsize, scene.psep)
        if not self.h:
            raise ValueError("grid dimensions inconsistent (Nx*Ny*Nz != numNodes)")
        pos = np.ascontiguousarray(scene.pos, np.float64)
        mat = np.ascontiguousarray(scene.mat, np.int32)
        obj = np.ascontiguousarray(scene.obj, np.int32)
        self._call("add_particles", self.h, scene.n, _dp(pos), _ip(mat), _ip(obj))
        vel = scene.vel
        for p in np.nonzero(np.any(vel != 0.0, axis=1))[0]:
            self._call("set_particle_vel", self.h, int(p), *map(float, vel[p]))
        st = scene.stress
        for p in np.nonzero(np.any(st != 0.0, axis=1))[0]:
            s6 = np.ascontiguousarray(st[p], np.float64)
            self._call("set_particle_stress", self.h, int(p), _dp(s6))
        for p in np.nonzero(scene.hold)[0]:
            self._call("hold_particle", self.h, int(p))
        for p in np.nonzero(scene.pbc_type)[0]:
            v = np.ascontiguousarray(scene.pbc_val[p], np.float64)
            self._call("set_particle_bc", self.h, int(p), int(scene.pbc_type[p]), _dp(v), 4)
        temp = getattr(scene, "temp", None)
        if temp is not None and np.any(temp != 0.0):
            self.set_temps(np.nonzero(temp)[0], temp[temp != 0.0])
        flaw = getattr(scene, "flaw", None)
        if flaw is not None and np.any(flaw != 1.0):
            if kind != "port":
                raise ValueError("the reference has no per-particle flaw strains (only the restatement)")
            ids = np.nonzero(flaw != 1.0)[0].astype(np.int32)
            w = np.ascontiguousarray(flaw[ids], np.float64)
            self.lib.gyo_set_particle_flaws(self.h, int(ids.size), _ip(ids), _dp(w))
        for n in np.nonzero(scene.node_bc_type)[0]:
            v = np.ascontiguousarray(scene.node_bc_val[n], np.float64)
            self._call("set_node_bc", self.h, int(n), int(scene.node_bc_type[n]), _dp(v), 4)
        self._params = make_params(scene)
        self._mats = make_materials(scene.materials)
        rc = self._call("init_solver", self.h, C.byref(self._params), len(scene.materials), self._mats)
        if rc != 0:
            raise ValueError("material id out of range")
        if scene.dt is not None:
            self._call("set_dt", self.h, float(scene.dt))
        self.dt = self._call("get_dt", self.h)
        self.step_index = 0
        self.t = 0.0

    def set_temps(self, ids, T) -> None:
        """MaterialPoints::setTemp for particles given by their original index."""
        ids = np.ascontiguousarray(ids, np.int32)
        T = np.ascontiguousarray(T, np.float64)
        self._call("set_particle_temps", self.h, int(ids.size), _ip(ids), _dp(T))

    def _call(self, name, *args):
        return getattr(self.lib, self.pre + name)(*args)

    def close(self):
        if self.h:
            self._call("destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, t: Optional[float] = None, step: Optional[int] = None) -> None:
        """One iterate_CPU(t, step) with the script loop's convention t = step*dt."""
        s = self.step_index if step is None else step
        tt = s * self.dt if t is None else t
        if self.kind == "port":
            rc = self._call("step", self.h, float(tt), int(s))
        else:
            rc = self._call("step", self.h, float(tt), int(s), int(self.mode))
        if rc != 0:
            raise RuntimeError("oracle step failed: a particle left the indexable cell range")
        self.step_index = s + 1
        self.t = tt

    def run(self, nsteps: int) -> None:
        for _ in range(nsteps):
            self.step()

    # ---- access ------------------------------------------------------------------------
    @property
    def n(self) -> int:
        return self._call("num_particles", self.h)

    def pfield(self, name: str, by_id: bool = True) -> np.ndarray:
        w = P_WIDTH[name]
        out = np.empty((self.n, w), np.float64)
        self._call("get_particle_field", self.h, P_FIELDS[name], _dp(out))
        if by_id:
            out = out[np.argsort(self.pifield("pid", by_id=False), kind="stable")]
        return out if w > 1 else out[:, 0]

    def pifield(self, name: str, by_id: bool = True) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        self._call("get_particle_ifield", self.h, PI_FIELDS[name], _ip(out))
        if by_id and name != "pid":
            out = out[np.argsort(self.pifield("pid", by_id=False), kind="stable")]
        return out

    def nfield(self, name: str) -> np.ndarray:
        nn = self._call("num_nodes", self.h)
        w = 1 if name.startswith("mass") or name.startswith("temp") else 3
        out = np.empty((nn, w), np.float64)
        self._call("get_node_field", self.h, N_FIELDS[name], _dp(out))
        return out if w > 1 else out[:, 0]

    def nifield(self, name: str) -> np.ndarray:
        nn = self._call("num_nodes", self.h)
        w = 2 if name in ("body", "rigid") else 1
        out = np.empty(nn * w, np.int32)
        self._call("get_node_ifield", self.h, NI_FIELDS[name], _ip(out))
        return out.reshape(nn, w) if w > 1 else out


def gimp_shape(dist, h, lp):
    lib, _ = _lib("port")
    return lib.gyo_gimp_shape(float(dist), float(h), float(lp))


def gimp_grad(dist, h, lp, xp):
    lib, _ = _lib("port")
    return lib.gyo_gimp_grad(float(dist), float(h), float(lp), float(xp))


def sym_eigen(a):
    lib, _ = _lib("port")
    a = np.ascontiguousarray(a, np.float64).reshape(9)
    V = np.empty(9)
    d = np.empty(3)
    lib.gyo_sym_eigen(_dp(a), _dp(V), _dp(d))
    return d, V.reshape(3, 3)
