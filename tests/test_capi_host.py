"""The C-ABI library on the host (no GPU compute): symbols, setters, pattern."""
import ctypes

import numpy as np
import pytest

import oracle
from plugin_navierstokes_gb300 import NavierStokesFV1, NSFV1Error, _capi, mesh, mesh_pattern


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    syms = _capi.header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s


def test_setters_string_ids_and_errors():
    d = NavierStokesFV1("u,v,p", "Inner")
    assert d.dim == 2 and d.disc_type() == "fv1"
    for name in ["no", "FULL", " lps ", "LinearProfileSkewed", "skewed", "positive", " POS"]:
        d.set_upwind(name)
    with pytest.raises(NSFV1Error) as ex:
        d.set_upwind("weighted")
    assert ex.value.status == _capi.ERR_ARGUMENT and "not found" in str(ex.value)
    # the positive upwind's workspace comes with the first device use, not with the setter
    d.set_stabilization("flow")
    d.set_stabilization_upwind("pos")
    for name in ["fields", "Flow", "without"]:
        d.set_stabilization(name)
    d.set_stabilization("fields", "FivePoint")
    with pytest.raises(NSFV1Error):
        d.set_stabilization("supg")
    with pytest.raises(NSFV1Error):
        d.set_stabilization("fields", "bogus")
    with pytest.raises(NSFV1Error):
        d.set_source([1.0, 2.0, 3.0])
    d.set_source([1.0, 2.0])
    with pytest.raises(NSFV1Error):
        NavierStokesFV1("u,v,w,p,q")


def test_assembly_without_setup_is_a_state_error():
    d = NavierStokesFV1("u,v,p")
    lib = _capi.load()
    st = lib.nsfv1_assemble_defect(d._h, None, None, 0.0, None, None)
    assert st == _capi.ERR_STATE


def test_linear_algebra_entry_points_check_their_arguments_on_the_host():
    """The linear-solve and split-SpMV entry points refuse a handle without a
    mesh and invalid arguments before any device work."""
    d = NavierStokesFV1("u,v,p")
    lib = _capi.load()
    p = _capi.NewtonParams(1e-8, 0.0, 10, 1e-4, 100, 0, _capi.F64, _capi.BICGSTAB, 30)
    it, rr, rs = ctypes.c_int(-1), ctypes.c_double(-1.0), ctypes.c_int(-1)
    st = lib.nsfv1_linear_solve(d._h, None, None, None, ctypes.byref(p), ctypes.byref(it), ctypes.byref(rr), ctypes.byref(rs), None)
    assert st == _capi.ERR_STATE and "no mesh" in lib.nsfv1_last_error(d._h).decode()
    assert it.value == -1 and rs.value == -1   # outputs untouched on refusal
    assert lib.nsfv1_linear_solve(None, None, None, None, ctypes.byref(p), None, None, None, None) == _capi.ERR_ARGUMENT
    assert lib.nsfv1_bsr_mv_split(d._h, None, None, None, None) == _capi.ERR_STATE
    assert lib.nsfv1_split_vector(-1, None, None, None) == _capi.ERR_ARGUMENT
    assert lib.nsfv1_split_vector(0, None, None, None) == _capi.OK   # nothing to do
    assert lib.nsfv1_split_vector(4, None, None, None) == _capi.ERR_ARGUMENT


@pytest.mark.parametrize("gen", ["quads", "hexes", "tris"])
def test_pattern_and_coloring_bit_exact_with_oracle(gen):
    roid, X, C = {"quads": lambda: mesh.structured_quads(7), "hexes": lambda: mesh.structured_hexes(4),
                  "tris": lambda: mesh.jittered_triangles(6)}[gen]()
    rp, ci, col, nc = mesh_pattern(roid, X.shape[0], C)
    o = oracle.Oracle(X.shape[1])
    o.set_mesh(roid, X, C)
    orp, oci = o.pattern()
    ocol, onc = o.coloring()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.array_equal(col, ocol) and nc == onc


def test_pattern_rejects_bad_connectivity():
    roid, X, C = mesh.structured_quads(2)
    C = C.copy(); C[0, 0] = 99
    with pytest.raises(NSFV1Error):
        mesh_pattern(roid, X.shape[0], C)


@pytest.mark.parametrize("roid", [2, 3, 4, 8])
def test_reference_tables_match_oracle(roid):
    lib = _capi.load()
    nco, ne, ns = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    edges = np.zeros(24, np.int32); snc = np.zeros(6, np.int32); sides = np.zeros(24, np.int32); ef = np.zeros(24, np.int32)
    assert lib.nsfv1_ref_tables(roid, ctypes.byref(nco), ctypes.byref(ne), edges.ctypes.data, ctypes.byref(ns),
                                snc.ctypes.data, sides.ctypes.data, ef.ctypes.data) == 0
    t = oracle.ref_tables(roid)
    assert nco.value == t["nco"]
    assert np.array_equal(edges[:2 * ne.value].reshape(-1, 2), t["edges"])
    assert np.array_equal(snc[:ns.value], t["side_nco"])
    for s in range(ns.value):
        assert np.array_equal(sides[4 * s:4 * s + snc[s]], t["sides"][s][:snc[s]])
    if roid in (4, 8):
        assert np.array_equal(ef[:2 * ne.value].reshape(-1, 2), t["edge_face"])


def test_cavity_dirichlet_rows():
    roid, X, C = mesh.structured_quads(4)
    dofs, vals = mesh.cavity_dirichlet(X, 2.0)
    b = 3
    nodes = dofs // b
    assert np.all(np.diff(dofs) > 0)
    assert (0 * b + 2) in dofs.tolist()
    lid = [(n, v) for d, n, v in zip(dofs, nodes, vals) if d % b == 0 and v != 0]
    assert all(abs(X[n, 1] - 1) < 1e-12 and 0 < X[n, 0] < 1 for n, _ in lid) and len(lid) == 3


def test_empty_and_oversized_meshes_are_rejected_before_any_device_work():
    lib = _capi.load()
    d = NavierStokesFV1("u,v,w,p")
    coords = np.zeros((8, 3))
    conn = np.arange(8, dtype=np.int32)
    # no elements / no nodes
    assert lib.nsfv1_set_mesh(d._h, _capi.HEXAHEDRON, 8, coords.ctypes.data, 0, conn.ctypes.data) == _capi.ERR_ARGUMENT
    assert lib.nsfv1_set_mesh(d._h, _capi.HEXAHEDRON, 0, coords.ctypes.data, 1, conn.ctypes.data) == _capi.ERR_ARGUMENT
    # 32-bit index limits (checked from the sizes alone, the arrays are not read)
    assert lib.nsfv1_set_mesh(d._h, _capi.HEXAHEDRON, 8, coords.ctypes.data, 1 << 26, conn.ctypes.data) == _capi.ERR_ARGUMENT
    assert "32-bit" in d.last_error()
    # unknown element type
    assert lib.nsfv1_set_mesh(d._h, 7, 8, coords.ctypes.data, 1, conn.ctypes.data) == _capi.ERR_ARGUMENT


def test_single_element_pattern_and_ragged_coloring():
    # one hexahedron: a dense 8 x 8 block pattern, one colour
    rp, ci, col, nc = mesh_pattern(_capi.HEXAHEDRON, 8, np.arange(8, dtype=np.int32)[None, :])
    assert np.array_equal(rp, np.arange(9) * 8) and nc == 1 and col.tolist() == [0]
    # a ragged strip of triangles sharing one node (a fan): every element needs its own colour
    fan = np.array([[0, k, k + 1] for k in range(1, 7)], np.int32)
    rp, ci, col, nc = mesh_pattern(_capi.TRIANGLE, 8, fan)
    assert nc == 6 and sorted(col.tolist()) == list(range(6))
    o = oracle.Oracle(2)
    X = np.zeros((8, 2))
    X[1:, 0] = np.cos(np.linspace(0, 3, 7))
    X[1:, 1] = np.sin(np.linspace(0, 3, 7))
    o.set_mesh(_capi.TRIANGLE, X, fan)
    orp, oci = o.pattern()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


def test_meshes_with_unreferenced_nodes_are_rejected():
    """A node that no element references would get a matrix row without a diagonal
    block: nsfv1_set_mesh and nsfv1_mesh_pattern refuse such meshes (before any
    device work)."""
    lib = _capi.load()
    roid, X, C = mesh.structured_quads(3)
    Xo = np.vstack([X, [[2.0, 2.0]]])   # one orphan node after the grid
    d = NavierStokesFV1("u,v,p")
    st = lib.nsfv1_set_mesh(d._h, roid, Xo.shape[0], np.ascontiguousarray(Xo).ctypes.data, C.shape[0],
                            np.ascontiguousarray(C, dtype=np.int32).ctypes.data)
    assert st == _capi.ERR_ARGUMENT and "belongs to no element" in d.last_error()
    with pytest.raises(NSFV1Error):
        mesh_pattern(roid, Xo.shape[0], C)


def test_pattern_and_coloring_bit_exact_at_benchmark_size_host():
    """The 64^3 hexahedral benchmark mesh through the host-only pattern build:
    7,189,057 blocks and the element colouring, bit-exact with the oracle."""
    roid, X, C = mesh.structured_hexes(64)
    rp, ci, col, nc = mesh_pattern(roid, X.shape[0], C)
    o = oracle.Oracle(3)
    o.set_mesh(roid, X, C)
    orp, oci = o.pattern()
    ocol, onc = o.coloring()
    assert ci.size == 193 ** 3 and nc == onc == 8
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci) and np.array_equal(col, ocol)


def test_pac_upwind_needs_an_upwind_and_a_stabilisation():
    """set_pac_upwind(true) (navier_stokes_fv1.h:217-225) with the reference's texts."""
    d = NavierStokesFV1("u,v,p")
    with pytest.raises(NSFV1Error) as ex:
        d.set_pac_upwind(True)
    assert ex.value.status == _capi.ERR_STATE and "Upwind must be specified previously" in str(ex.value)
    d.set_upwind("full")
    with pytest.raises(NSFV1Error) as ex:
        d.set_pac_upwind(True)
    assert "Stabilization must be specified previously" in str(ex.value)
    d.set_stabilization("fields")
    d.set_pac_upwind(True)
    d.set_pac_upwind(False)   # changes nothing, as in the reference


def test_bounds_checked_assembly_compiles(tmp_path):
    """The NSFV1_BOUNDS_CHECK variant of the assembly kernels (index checks that set
    an error bit instead of trapping) builds for sm_103a."""
    from plugin_navierstokes_gb300 import build

    objs = build.compile_bounds_checked(tmp_path / "assemble_bc.o")
    assert len(objs) == len(build.BOUNDS_CHECKED_SOURCES)
    assert all(o.exists() and o.stat().st_size > 0 for o in objs)
