"""ctypes binding of libgraphyt_gpu.so (include/graphyt_gpu.h).

The library is built in-tree by :mod:`graphyt_gb300.build`.  Loading fails loudly when it
is missing: there is no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgraphyt_gpu.so")

GY_SORT_STATIC_MAX = 262144

GY_OK, GY_ERR_ARG, GY_ERR_CUDA, GY_ERR_STATE, GY_ERR_RANGE, GY_ERR_UNSUPPORTED, GY_ERR_NONFINITE, GY_ERR_NOMEM = (
    0, -1, -2, -3, -4, -5, -6, -7)
STATUS_NAMES = {0: "GY_OK", -1: "GY_ERR_ARG", -2: "GY_ERR_CUDA", -3: "GY_ERR_STATE", -4: "GY_ERR_RANGE",
                -5: "GY_ERR_UNSUPPORTED", -6: "GY_ERR_NONFINITE", -7: "GY_ERR_NOMEM"}

P_FIELDS = dict(pos=0, pos0=1, disp=2, vel=3, stress=4, strain=5, pstrain=6, eqps=7, damage=8, smax=9,
                mass=10, density=11, volume=12, normals=13, temp=14, tempgrad=15)
P_WIDTH = dict(pos=3, pos0=3, disp=3, vel=3, stress=6, strain=6, pstrain=6, eqps=1, damage=1, smax=1,
               mass=1, density=1, volume=1, normals=3, temp=1, tempgrad=3)
PI_FIELDS = dict(cellid=0, material=1, object=2, device_slot=3)
N_FIELDS = dict(mass=0, vel=1, force=2, vel1=3, acc1=4)


class GridDesc(C.Structure):
    _fields_ = [("L", C.c_double * 3), ("cellsize", C.c_double), ("psep", C.c_double)]


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


class Options(C.Structure):
    _fields_ = [("sort_every", C.c_int), ("full_sort", C.c_int), ("use_graph", C.c_int),
                ("track_normals", C.c_int), ("check_finite", C.c_int), ("keep_node_fields", C.c_int),
                ("p2g_lanes", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("mass", C.c_double), ("momentum", C.c_double * 3), ("kinetic", C.c_double),
                ("strain_energy", C.c_double), ("active_nodes", C.c_int64), ("steps", C.c_int64),
                ("status_flags", C.c_int64)]


# every entry point of include/graphyt_gpu.h with its ctypes signature
_vp, _dp, _ip, _i64p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int64)
SIGNATURES = {
    "gy_abi_version": (C.c_int, []),
    "gy_create": (C.c_int, [C.POINTER(GridDesc), C.c_int, C.POINTER(C.c_void_p)]),
    "gy_destroy": (C.c_int, [_vp]),
    "gy_last_error": (C.c_char_p, [_vp]),
    "gy_grid_dims": (C.c_int, [_vp, _ip, _i64p]),
    "gy_add_particles": (C.c_int, [_vp, C.c_int64, _dp, _ip, _ip]),
    "gy_set_particle_vel": (C.c_int, [_vp, C.c_int64, _i64p, _dp]),
    "gy_set_particle_stress": (C.c_int, [_vp, C.c_int64, _i64p, _dp]),
    "gy_set_particle_damage": (C.c_int, [_vp, C.c_int64, _i64p, _dp]),
    "gy_set_particle_flaw": (C.c_int, [_vp, C.c_int64, _i64p, _dp]),
    "gy_tc_gemm_bf16": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp]),
    "gy_tc_wait_check": (C.c_int, [_vp, _vp, _vp]),
    "gy_mlp_param_count": (C.c_int64, []),
    "gy_mlp_forward": (C.c_int, [_vp, _vp, C.c_int64, _vp, _vp, _vp]),
    "gy_mlp_grad": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp]),
    "gy_dp_log_begin": (C.c_int, [_vp, C.c_int64, C.c_int]),
    "gy_dp_log_end": (C.c_int, [_vp]),
    "gy_dp_log_count": (C.c_int, [_vp, _i64p]),
    "gy_dp_log_read": (C.c_int, [_vp, _vp, _vp, C.c_int64]),
    "gy_dp_surrogate_train": (C.c_int, [_vp, C.c_int, C.c_int, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "gy_set_dp_surrogate": (C.c_int, [_vp, _vp, C.c_int, C.c_float]),
    "gy_get_dp_surrogate": (C.c_int, [_vp, _vp]),
    "gy_dp_surrogate_counts": (C.c_int, [_vp, _i64p, _i64p]),
    "gy_mlp_train": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64, C.c_int,
                               C.POINTER(C.c_float), _vp, _vp]),
    "gy_set_particle_temp": (C.c_int, [_vp, C.c_int64, _i64p, _dp]),
    "gy_hold_particles": (C.c_int, [_vp, C.c_int64, _i64p]),
    "gy_set_particle_bc": (C.c_int, [_vp, C.c_int64, _i64p, _ip, _dp]),
    "gy_set_node_bc": (C.c_int, [_vp, C.c_int64, _i64p, _ip, _dp]),
    "gy_initialize": (C.c_int, [_vp, C.POINTER(Material), C.c_int, C.POINTER(Params)]),
    "gy_set_dt": (C.c_int, [_vp, C.c_double]),
    "gy_get_dt": (C.c_int, [_vp, _dp]),
    "gy_set_params": (C.c_int, [_vp, C.POINTER(Params)]),
    "gy_set_options": (C.c_int, [_vp, C.POINTER(Options)]),
    "gy_get_options": (C.c_int, [_vp, C.POINTER(Options)]),
    "gy_step": (C.c_int, [_vp, C.c_double, C.c_int]),
    "gy_steps": (C.c_int, [_vp, C.c_double, C.c_int, C.c_int, C.c_int]),
    "gy_sync": (C.c_int, [_vp]),
    "gy_stream": (C.c_void_p, [_vp]),
    "gy_num_particles": (C.c_int, [_vp, _i64p]),
    "gy_get_particles": (C.c_int, [_vp, C.c_int, _dp, C.c_int64]),
    "gy_get_particles_int": (C.c_int, [_vp, C.c_int, _ip, C.c_int64]),
    "gy_get_nodes": (C.c_int, [_vp, C.c_int, _dp, C.c_int64]),
    "gy_sort_keys": (C.c_int, [_ip, C.c_int64, _ip, C.c_int]),
    "gy_resort_keys": (C.c_int, [_ip, _ip, C.c_int64, _ip, _ip, C.c_int]),
    "gy_state_size": (C.c_int, [_vp, _i64p]),
    "gy_state_save": (C.c_int, [_vp, C.c_void_p, C.c_int64]),
    "gy_state_load": (C.c_int, [_vp, C.c_void_p, C.c_int64]),
    "gy_sort_keys_static": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p]),
    "gy_get_stats": (C.c_int, [_vp, C.POINTER(Stats)]),
    "gy_set_phase_timing": (C.c_int, [_vp, C.c_int]),
    "gy_get_phase_times": (C.c_int, [_vp, C.POINTER(C.c_float), _i64p]),
    "gy_time_steps": (C.c_int, [_vp, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "gy_kernel_launches": (C.c_int64, []),
}

_lib = None


class GraphytGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load the CUDA library; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m graphyt_gb300.build` "
                          "(this package has no CPU fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, handle=None, what: str = ""):
    if rc != GY_OK:
        msg = load().gy_last_error(handle).decode() if handle else ""
        raise GraphytGPUError(rc, f"{what} {msg}".strip())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def sort_keys(keys) -> np.ndarray:
    """Stable device sort of non-negative int keys; returns the permutation."""
    k = np.ascontiguousarray(keys, np.int32)
    out = np.empty(len(k), np.int32)
    check(load().gy_sort_keys(iptr(k), len(k), iptr(out), -1), None, "gy_sort_keys")
    return out


def resort_keys(keys, prev_sorted):
    """Incremental device re-sort (the step's sort after its first): keys[i] is the current
    key of the particle whose key at the last sort was prev_sorted[i] (non-decreasing).
    Returns (perm, sorted keys), equal to the stable sort of keys."""
    k = np.ascontiguousarray(keys, np.int32)
    p = np.ascontiguousarray(prev_sorted, np.int32)
    if len(k) != len(p):
        raise ValueError("keys and prev_sorted differ in length")
    perm = np.empty(len(k), np.int32)
    srt = np.empty(len(k), np.int32)
    check(load().gy_resort_keys(iptr(k), iptr(p), len(k), iptr(perm), iptr(srt), -1), None, "gy_resort_keys")
    return perm, srt
