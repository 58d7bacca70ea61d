"""Host side of the boundary, no GPU: the ctypes layouts against the C header, the BC codes
against the kernels' enum, and the Python mirror of the reference's classes (defaults,
grid sizes, node order, setter semantics)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from graphyt_gb300 import _lib as L
from graphyt_gb300 import graphyt
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "include")
REF_BC_HEADER = os.path.join(oracle.REFERENCE_DIR, "BoundaryConditions.hpp")

_STRUCTS = {
    "gy_grid_desc": L.GridDesc, "gy_material": L.Material, "gy_params": L.Params,
    "gy_options": L.Options, "gy_stats": L.Stats,
}
_ENUMS = ["GY_OK", "GY_ERR_ARG", "GY_ERR_CUDA", "GY_ERR_STATE", "GY_ERR_RANGE", "GY_ERR_UNSUPPORTED",
          "GY_ERR_NONFINITE", "GY_ERR_NOMEM", "GY_SORT_STATIC_MAX", "GY_ABI_VERSION", "GY_P_NFIELDS",
          "GY_N_NFIELDS"] + ["GY_P_" + k.upper() for k in L.P_FIELDS] + \
         ["GY_PI_" + k.upper() for k in L.PI_FIELDS] + ["GY_N_" + k.upper() for k in L.N_FIELDS]


def _header_layout(tmp_path):
    """Compile a probe against include/graphyt_gpu.h and read sizes, offsets and constants."""
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "graphyt_gpu.h"', "int main(void) {"]
    for cname, cls in _STRUCTS.items():
        lines.append(f'printf("size {cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("off {cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    for e in _ENUMS:
        lines.append(f'printf("const {e} %lld\\n", (long long)({e}));')
    lines += ["return 0; }"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", HEADER_DIR, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict((k, int(v)) for k, v in (ln.rsplit(" ", 1) for ln in out.splitlines()))


def test_ctypes_layouts_and_constants_match_header(tmp_path):
    got = _header_layout(tmp_path)
    for cname, cls in _STRUCTS.items():
        assert got[f"size {cname}"] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[f"off {cname}.{fname}"] == getattr(cls, fname).offset, (cname, fname)
    py = {"GY_OK": L.GY_OK, "GY_ERR_ARG": L.GY_ERR_ARG, "GY_ERR_CUDA": L.GY_ERR_CUDA,
          "GY_ERR_STATE": L.GY_ERR_STATE, "GY_ERR_RANGE": L.GY_ERR_RANGE,
          "GY_ERR_UNSUPPORTED": L.GY_ERR_UNSUPPORTED, "GY_ERR_NONFINITE": L.GY_ERR_NONFINITE,
          "GY_ERR_NOMEM": L.GY_ERR_NOMEM, "GY_SORT_STATIC_MAX": L.GY_SORT_STATIC_MAX,
          "GY_P_NFIELDS": len(L.P_FIELDS), "GY_N_NFIELDS": len(L.N_FIELDS)}
    py.update({"GY_P_" + k.upper(): v for k, v in L.P_FIELDS.items()})
    py.update({"GY_PI_" + k.upper(): v for k, v in L.PI_FIELDS.items()})
    py.update({"GY_N_" + k.upper(): v for k, v in L.N_FIELDS.items()})
    for name, value in py.items():
        assert got[f"const {name}"] == value, name
    # every status the header defines has a name for error messages
    assert set(L.STATUS_NAMES) == {got[f"const {n}"] for n in _ENUMS[:8]}


def test_bc_codes_match_kernel_enum():
    """Every BCTypes value the kernels act on (gy_common.cuh) has the same number in Python."""
    src = open(os.path.join(ROOT, "graphyt_gb300", "csrc", "gy_common.cuh")).read()
    body = re.search(r"enum BCType : int \{(.*?)\};", src, re.S).group(1)
    pairs = re.findall(r"BC_([A-Z_]+)\s*=\s*(\d+)", body)
    assert len(pairs) >= 15
    for name, value in pairs:
        assert getattr(graphyt.BCTypes, name.lower()) == int(value), name


@pytest.mark.skipif(not os.path.isfile(REF_BC_HEADER), reason="reference tree not available")
def test_bc_types_follow_reference_enum():
    """BCTypes::function (BoundaryConditions.hpp:6-77), names in declaration order."""
    text = open(REF_BC_HEADER).read()
    body = re.search(r"enum\s+function\s*\{(.*?)\}", text, re.S).group(1)
    names = [n.strip() for n in re.sub(r"//[^\n]*", "", body).split(",") if n.strip()]
    assert names == graphyt._BC_NAMES
    for i, n in enumerate(names):
        assert getattr(graphyt.BCTypes, n) == i


def test_material_defaults_and_ctype():
    """MaterialModels::MaterialModels (MaterialModels.cpp:4-26) defaults, and the struct the
    library receives carries every field."""
    m = graphyt.MaterialModels()
    want = dict(bulkMod=1e7, shearMod=5000.0, density=1000.0, isRigid=False, viscosity=1.0,
                thermalConductivity=391.0, specificHeatCapacity=385.2, yieldStress=1e7, phi=40.0,
                psi=10.0, cohesion=1e5, criticalStrain=0.01, isDamage=False, damageModel=1, Cg=586.52,
                damageM=9.0, damageK=5.39e36, turbStress=1e10, model=1)
    for k, v in want.items():
        assert getattr(m, k) == v, k
    m.setBulkMod(3e10); m.setShearMod(2e10); m.setFrictionAngle(30); m.setDilatancyAngle(0)
    m.setIsRigid(1.0); m.setIsDamage(True); m.setModel(4); m.setCrackSpeed(1867.4)
    c = m._ctype()
    assert (c.bulkMod, c.shearMod, c.phi, c.psi, c.Cg) == (3e10, 2e10, 30.0, 0.0, 1867.4)
    assert (c.isRigid, c.isDamage, c.model, c.damageModel) == (1, 1, 4, 1)
    assert {f for f, _ in L.Material._fields_} == set(L.MAT_DOUBLE_FIELDS) | set(L.MAT_INT_FIELDS)


def test_parameters_ctype():
    """Parameters(tmax, is3D) (Parameters.cpp:8-15) and its setters reach the library struct."""
    p = graphyt.Parameters(0.5, True)
    assert (p.CFL, p.mu, p.velocityDampingCoef) == (0.1, 0.0, 0.0)
    p.setGravity(0, 0, -9.81); p.setDampingCoef(0.2); p.setCFL(0.3); p.setFriction(0.4)
    p.setFixedGridBCs(True)
    c = p._ctype()
    assert list(c.gravity) == [0.0, 0.0, -9.81]
    assert (c.damping, c.CFL, c.mu, c.tmax, c.is3D, c.fixed_grid_bcs) == (0.2, 0.3, 0.4, 0.5, 1, 1)


def test_nodes_sizes_and_order():
    """Nodes(L, cellsize): Nx truncated, numNodes rounded (Nodes.cpp:12, 71-73); node n at
    (i, j, k) with n = i + Nx (j + Ny k) (the k, j, i loop of Nodes.cpp:76-90)."""
    n = graphyt.Nodes([1.0, 1.0, 1.0], 0.05)
    assert (n.Nx, n.Ny, n.Nz, n.numNodes) == (21, 21, 21, 9261)
    n = graphyt.Nodes([4.0, 2.0, 2.0], 0.01)
    assert (n.Nx, n.Ny, n.Nz, n.numNodes) == (401, 201, 201, 401 * 201 * 201)
    n = graphyt.Nodes([0.3, 0.2, 0.1], 0.1)  # 0.3 / 0.1 = 2.9999999999999996 in binary
    assert n.Nx == 3 and n.numNodes == round(4.0 * 3 * 2)
    assert n.Nx * n.Ny * n.Nz != n.numNodes  # the grid gy_create rejects
    n = graphyt.Nodes([1.0, 0.5, 0.75], 0.25)
    pos = n.getPosArr().reshape(-1, 3)
    assert len(pos) == n.numNodes
    for idx in (0, 1, n.Nx, n.Nx * n.Ny, n.numNodes - 1, 37):
        i, j, k = idx % n.Nx, (idx // n.Nx) % n.Ny, idx // (n.Nx * n.Ny)
        assert np.allclose(pos[idx], [i * 0.25, j * 0.25, k * 0.25])
        assert (n.getPosX(idx), n.getPosY(idx), n.getPosZ(idx)) == tuple(pos[idx])
    assert not n.getMassArr().any() and n.getVelArr().shape == (3 * n.numNodes,)


def test_node_and_particle_bcs_write_only_given_values():
    """Nodes::setBC and MaterialPoints::setBC (Nodes.cpp:155-163, MaterialPoints.cpp:88-93)
    write the type and the values given; the other values stay as they were."""
    n = graphyt.Nodes([0.2, 0.2, 0.2], 0.05)
    n.setBC(7, graphyt.BCTypes.grid_vx_vy, [1.0, 2.0, 3.0, 4.0])
    n.setBC(7, graphyt.BCTypes.grid_vx, [9.0])
    assert n._bc_type[7] == graphyt.BCTypes.grid_vx
    assert list(n._bc_val[7]) == [9.0, 2.0, 3.0, 4.0]
    n.setBCs([1, 2], graphyt.BCTypes.grid_vy, [[5.0], [6.0]])
    assert list(n._bc_val[[1, 2], 0]) == [5.0, 6.0] and (n._bc_type[[1, 2]] == 2).all()

    mp = graphyt.MaterialPoints(n)
    mp.addPyckGeom(np.arange(12, dtype=float) * 0.01, 4)
    mp.add(4, 0.1, 0.1, 0.1)
    assert mp.numParticles == 5
    mp.setBC(3, graphyt.BCTypes.mp_vxsin, [0.5, 2.0])
    assert mp._bc[3] == (graphyt.BCTypes.mp_vxsin, [0.5, 2.0, 0.0, 0.0])
    mp.setBC(3, graphyt.BCTypes.mp_vx, [0.1])
    assert mp._bc[3] == (graphyt.BCTypes.mp_vx, [0.1, 2.0, 0.0, 0.0])
    mp.setBCs([0, 1], graphyt.BCTypes.mp_vz, [-0.1])
    assert mp._bc[0] == mp._bc[1] == (graphyt.BCTypes.mp_vz, [-0.1, 0.0, 0.0, 0.0])


def test_particle_ids_and_getters_before_the_solver():
    """Material and object ids are host arrays until a Solver exists; float state getters
    say that the state lives on the GPU."""
    n = graphyt.Nodes([0.2, 0.2, 0.2], 0.05)
    mp = graphyt.MaterialPoints(n)
    mp.addPyckGeom(np.zeros(9), 3)
    assert list(mp.getMatArr()) == [0, 0, 0]
    mp.setMaterialID(1, 2)
    mp.addPyckIntField(graphyt._IntField("objectID", [4, 5, 6, 7]))
    assert list(mp.getMatArr()) == [0, 2, 0] and list(mp.getObjectIDArr()) == [4, 5, 6]
    assert mp.getMatID(1) == 2 and mp.getObjID(2) == 6
    with pytest.raises(RuntimeError):
        mp.getStressArr()


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    """Without the built CUDA library the package raises; there is no CPU path to fall to."""
    monkeypatch.setattr(L, "_lib", None)
    with pytest.raises(ImportError, match="no CPU fallback"):
        L.load(str(tmp_path / "libgraphyt_gpu.so"))
