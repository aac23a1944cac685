"""CPU: the C-ABI library loads, exports what include/lbm_gb300.h declares,
and its host preprocessing takes the reference's CellIni decisions."""
import ctypes
import os
import re

import numpy as np
import pytest

import cases
import parallellbmcranfield_gb300 as G
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbm_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(G.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(G.EXPORTS) == syms


def test_status_strings():
    L = G.load()
    for s in range(7):
        assert L.lbm_status_string(s)
    assert L.lbm_status_string(99) == b"unknown status"


def reference_flags(ints, drag_id):
    """BRec flags from the reference's CellIni fields (ref_get_init layout)."""
    corner, boundary, bid = ints[:, 1], ints[:, 2], ints[:, 3]
    stream, bc = ints[:, 5:14], ints[:, 14:23]
    fl = np.zeros(len(ints), np.uint64)
    for k in range(9):
        fl |= (stream[:, k] == 1).astype(np.uint64) << np.uint64(k)
        fl |= (bc[:, k] == 1).astype(np.uint64) << np.uint64(9 + k)
    fl |= (((boundary == 2) & (bc[:, 2] == 2) & (corner != 1)).astype(np.uint64) << np.uint64(18))
    fl |= (((boundary == 2) & (bc[:, 3] == 2) & (corner != 1)).astype(np.uint64) << np.uint64(19))
    fl |= ((bc[:, 1] == 3).astype(np.uint64) << np.uint64(20))
    if drag_id:
        fl |= ((bid == drag_id).astype(np.uint64) << np.uint64(21))
    return fl


@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_preprocessing_matches_cellini(name):
    spec, params, start, steps = cases.ALL[name]
    mesh = cases.build_mesh(spec)
    port = O.Port(mesh.nodes, mesh.conns, **cases.oracle_params(params))
    ints, reals = port.init_fields()
    ins = G.inspect_mesh(mesh, **params)
    assert (ins["n"], ins["m"]) == (port.n, port.m)
    fluid = ints[:, 0] == 1
    assert np.array_equal(ins["cls"] > 0, fluid)
    sp = ins["cls"] == 3
    bulk = ins["cls"] == 1
    # bulk cells: no boundary link at all
    assert not (ints[bulk, 14:23] != 0).any()
    ref = reference_flags(ints, params.get("drag_lift_id", 0))
    assert np.array_equal(ins["flags"][sp].astype(np.uint64), ref[sp])
    assert np.array_equal(ins["q"][sp], reals[sp, :9])


def test_invalid_arguments_are_rejected_on_the_host():
    mesh = G.Mesh.cavity(8)
    with pytest.raises(G.LbmError) as e:
        G.Solver(mesh, collision_model=7)
    assert e.value.status == G.LBM_INVALID
    with pytest.raises(G.LbmError) as e:
        G.Solver(mesh, outlet_profile=9)
    assert e.value.status == G.LBM_INVALID


def test_fluid_on_the_border_is_rejected():
    mesh = G.Mesh.cavity(6)
    nodes = mesh.nodes.copy()
    nodes[3, 4] = 1.0  # a fluid cell in row 0
    with pytest.raises(G.LbmError) as e:
        G.inspect_mesh(G.Mesh(nodes, mesh.conns))
    assert e.value.status == G.LBM_INVALID


def test_outlet_extrapolation_source_must_not_be_outlet():
    mesh = G.Mesh.channel(8, 4)
    conns = mesh.conns.copy()
    n, m = mesh.shape
    # an extra outlet link on the cell west of an outlet cell
    extra = np.array([[7, 2, 1, 3, 0.5, 0.5, 3]], np.float32)
    bad = G.Mesh(mesh.nodes, np.vstack([conns, extra]))
    with pytest.raises(G.LbmError):
        G.inspect_mesh(bad, outlet_profile=2)
    G.inspect_mesh(bad, outlet_profile=1)  # fine without extrapolation


def test_mesh_file_round_trip(tmp_path):
    mesh = G.Mesh.channel(20, 8, [(6.0, 4.3, 2.1)])
    nf, cf = tmp_path / "n.dat", tmp_path / "c.dat"
    mesh.write(nf, cf)
    back = G.Mesh.read(nf, cf)
    assert np.array_equal(back.nodes, mesh.nodes)
    assert np.array_equal(back.conns, mesh.conns)
    nodes, conns = O.read_mesh(str(nf), str(cf))  # the reference's fscanf parsing
    assert np.array_equal(nodes, mesh.nodes) and np.array_equal(conns, mesh.conns)


def test_missing_mesh_file_is_io_error(tmp_path):
    with pytest.raises(G.LbmError) as e:
        G.Mesh.read(tmp_path / "none.dat", tmp_path / "none2.dat")
    assert e.value.status == G.LBM_IO


@pytest.mark.skipif(not os.path.isdir(os.path.join(O.REF_CASES, "coarse")),
                    reason="shipped meshes not present")
@pytest.mark.parametrize("case,side", [("coarse", 125), ("medium", 253)])
def test_generator_reproduces_shipped_cavity(case, side):
    """The generated cavity takes every CellIni decision the shipped mesh does."""
    d = os.path.join(O.REF_CASES, case, "Mesh")
    shipped = G.Mesh.read(f"{d}/D2node.dat", f"{d}/BCconnectors.dat")
    gen = G.Mesh.cavity(side)
    assert shipped.shape == gen.shape
    assert np.abs(shipped.nodes - gen.nodes).max() < 5e-6
    a = G.inspect_mesh(shipped, uavg=0.08, rho_ini=5.0)
    b = G.inspect_mesh(gen, uavg=0.08, rho_ini=5.0)
    assert np.array_equal(a["cls"], b["cls"])
    assert np.array_equal(a["flags"], b["flags"])
    assert np.abs(a["q"] - b["q"]).max() < 1e-4


def test_batch_arguments_are_checked_on_the_host():
    """A batch shares precision, model and pattern; the library refuses mixtures
    before any device work (CPU)."""
    base = dict(uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.05, inlet_profile=2,
                curved_boundaries=1, outlet_profile=2)
    mesh = G.Mesh.cavity(20)
    with pytest.raises(G.LbmError) as e:
        G.Batch([(mesh, dict(base, collision_model=1)), (mesh, dict(base, collision_model=3))])
    assert e.value.status == G.LBM_INVALID
    with pytest.raises(G.LbmError) as e:
        G.Batch([(mesh, dict(base, collision_model=2))], precision="bf16dev")
    assert e.value.status == G.LBM_INVALID


@pytest.mark.parametrize("side", [2, 3, 30, 125])
def test_numpy_cavity_equals_library_cavity(side):
    """oracle.meshgen (numpy, for the CPU legs of bench.py) writes the same
    node and link lines as lbm_mesh_cavity."""
    from oracle import meshgen

    lib = G.Mesh.cavity(side)
    nodes, conns, shape = meshgen.cavity(side)
    assert lib.shape == shape
    assert np.array_equal(lib.nodes, nodes)
    assert np.array_equal(lib.conns, conns)
