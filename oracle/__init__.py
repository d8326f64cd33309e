"""CPU oracle of the FV1 Navier-Stokes path (TEST INFRASTRUCTURE ONLY).

A scalar FP64 C++ restatement of the reference's algorithm (nsfv1_oracle.cpp),
used as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg. The product package never imports this module.
Parity status: pinned to the reference's own element callbacks, compiled from
the reference sources against a ugcore stand-in (oracle/ugshim, build_ref(),
tests/test_reference_pin.py); the ugcore pieces stay restated (see the header
of nsfv1_oracle.cpp).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import c_char_p, c_double, c_int, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "lib" / "libnsfv1_oracle.so"
_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "nsfv1_oracle.cpp"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-C", str(HERE), "-B" if force else "all"], check=True, capture_output=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        sig = {
            "ora_create": (c_void_p, [c_int]), "ora_destroy": (None, [c_void_p]), "ora_last_error": (c_char_p, [c_void_p]),
            "ora_set_kinematic_viscosity": (c_int, [c_void_p, c_double]), "ora_set_density": (c_int, [c_void_p, c_double]),
            "ora_set_source": (c_int, [c_void_p, c_void_p, c_int]), "ora_set_exact_jacobian": (c_int, [c_void_p, c_double]),
            "ora_set_stokes": (c_int, [c_void_p, c_int]), "ora_set_laplace": (c_int, [c_void_p, c_int]),
            "ora_set_peclet_blend": (c_int, [c_void_p, c_int]), "ora_set_upwind": (c_int, [c_void_p, c_char_p]),
            "ora_set_stabilization": (c_int, [c_void_p, c_char_p, c_char_p]),
            "ora_set_stabilization_upwind": (c_int, [c_void_p, c_char_p]),
            "ora_set_pac_upwind": (c_int, [c_void_p, c_int]),
            "ora_geometry": (c_int, [c_int, c_void_p, c_void_p]),
            "ora_ref_tables": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
            "ora_elem_batch": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_void_p]),
            "ora_set_mesh": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_int64, c_void_p]),
            "ora_nnz_blocks": (c_int64, [c_void_p]), "ora_num_colors": (c_int, [c_void_p]),
            "ora_pattern": (c_int, [c_void_p, c_void_p, c_void_p]), "ora_coloring": (c_int, [c_void_p, c_void_p]),
            "ora_set_dirichlet": (c_int, [c_void_p, c_int64, c_void_p, c_void_p]),
            "ora_assemble": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p, c_int]),
            "ora_newton": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_double, c_int, c_double, c_int, c_int, c_int, c_void_p]),
            "ora_bsr_mv": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
            "ora_add_wall": (c_int, [c_void_p, c_int64, c_void_p]),
            "ora_add_dirichlet": (c_int, [c_void_p, c_int64, c_void_p, c_void_p]),
            "ora_add_inflow": (c_int, [c_void_p, c_int64, c_int, c_void_p, c_void_p]),
            "ora_vorticity": (c_int, [c_void_p, c_void_p, c_void_p]),
            "ora_add_outflow": (c_int, [c_void_p, c_int64, c_int, c_void_p]),
            "ora_outflow_elem": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
            "ora_eval_points": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int, c_void_p]),
            "ora_export": (c_int, [c_void_p, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_double, c_int, c_int, c_void_p,
                                   c_void_p, c_void_p]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


NSH = {2: 3, 3: 4, 4: 4, 6: 6, 8: 8}
DIM = {2: 2, 3: 2, 4: 3, 6: 3, 8: 3}


class Oracle:
    """The oracle's element disc + mesh (mirrors the product's setters)."""

    def __init__(self, dim: int):
        self.lib = load()
        self.dim = dim
        self.h = self.lib.ora_create(dim)
        self.mesh = None

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ora_destroy(self.h)
            self.h = None

    def _c(self, st):
        if st != 0:
            raise RuntimeError(f"oracle error {st}: {self.lib.ora_last_error(self.h).decode()}")

    def set_kinematic_viscosity(self, v): self._c(self.lib.ora_set_kinematic_viscosity(self.h, float(v)))
    def set_density(self, v): self._c(self.lib.ora_set_density(self.h, float(v)))
    def set_exact_jacobian(self, v): self._c(self.lib.ora_set_exact_jacobian(self.h, float(v)))
    def set_stokes(self, v): self._c(self.lib.ora_set_stokes(self.h, int(bool(v))))
    def set_laplace(self, v): self._c(self.lib.ora_set_laplace(self.h, int(bool(v))))
    def set_peclet_blend(self, v): self._c(self.lib.ora_set_peclet_blend(self.h, int(bool(v))))
    def set_upwind(self, n): self._c(self.lib.ora_set_upwind(self.h, n.encode()))
    def set_stabilization_upwind(self, n): self._c(self.lib.ora_set_stabilization_upwind(self.h, n.encode()))
    def set_pac_upwind(self, on): self._c(self.lib.ora_set_pac_upwind(self.h, int(bool(on))))

    def set_source(self, f):
        a = np.ascontiguousarray(f, dtype=np.float64)
        self._c(self.lib.ora_set_source(self.h, a.ctypes.data, a.size))

    def set_stabilization(self, n, dl=None):
        self._c(self.lib.ora_set_stabilization(self.h, n.encode(), dl.encode() if dl else None))

    def elem_batch(self, roid, corners, u, u_old=None, dt=0.0, want=("defA", "jacA", "defM", "jacM", "rhs")):
        corners = np.ascontiguousarray(corners, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        ne = corners.shape[0]
        nloc = (DIM[roid] + 1) * NSH[roid]
        out = {}
        for k in ("defA", "defM", "rhs"):
            out[k] = np.zeros((ne, nloc)) if k in want else None
        for k in ("jacA", "jacM"):
            out[k] = np.zeros((ne, nloc * nloc)) if k in want else None
        uo = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
        self._c(self.lib.ora_elem_batch(self.h, roid, ne, corners.ctypes.data, u.ctypes.data, _p(uo), float(dt),
                                        _p(out["defA"]), _p(out["jacA"]), _p(out["defM"]), _p(out["jacM"]), _p(out["rhs"])))
        return {k: v for k, v in out.items() if v is not None}

    def add_outflow(self, sides):
        """NavierStokesNoNormalStressOutflowFV1 on the given boundary sides [n][nco]."""
        sides = np.ascontiguousarray(sides, np.int32)
        self._c(self.lib.ora_add_outflow(self.h, sides.shape[0], sides.shape[1], sides.ctypes.data))

    def outflow_elem(self, roid, corners, u, side_mask):
        """The outflow disc's local defect and Jacobian of n elements whose sides side_mask[e]
        (bit s = reference side s) lie on the outflow boundary."""
        corners = np.ascontiguousarray(corners, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        m = np.ascontiguousarray(side_mask, np.uint32)
        ne, nl = corners.shape[0], (DIM[roid] + 1) * NSH[roid]
        d, J = np.zeros((ne, nl)), np.zeros((ne, nl * nl))
        self._c(self.lib.ora_outflow_elem(self.h, roid, ne, corners.ctypes.data, u.ctypes.data, m.ctypes.data, d.ctypes.data, J.ctypes.data))
        return d, J

    def vorticity(self, U):
        """vorticityFV1 of the nodal state U[n_nodes * b] on the mesh: one value per node."""
        U = np.ascontiguousarray(U, np.float64).ravel()
        out = np.zeros(self.coords.shape[0])
        self._c(self.lib.ora_vorticity(self.h, U.ctypes.data, out.ctypes.data))
        return out

    def eval_points(self, U, points, fct):
        """Function fct of the nodal state at global points [n][dim] (NaN outside the mesh)."""
        U = np.ascontiguousarray(U, np.float64).ravel()
        pts = np.ascontiguousarray(points, np.float64)
        out = np.zeros(pts.shape[0])
        self._c(self.lib.ora_eval_points(self.h, U.ctypes.data, pts.shape[0], pts.ctypes.data, int(fct), out.ctypes.data))
        return out

    def export(self, which, roid, corners, u, u_old=None, dt=0.0, ip_kind=0, local_ips=None, derivs=True):
        """The disc's data export `which` (EXPORTS index) of n elements: (values [n][nip][vs],
        derivatives [n][nip][b][nsh][vs] or None); ip_kind 0: SCVF ips, 1: SCV ips, 2: local_ips."""
        corners = np.ascontiguousarray(corners, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        lips = None if local_ips is None else np.ascontiguousarray(local_ips, np.float64)
        ne, nip, vs, b = corners.shape[0], export_nip(roid, ip_kind, lips), export_size(which, roid), DIM[roid] + 1
        val = np.zeros((ne, nip, vs))
        der = np.zeros((ne, nip, b, NSH[roid], vs)) if derivs else None
        uo = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
        self._c(self.lib.ora_export(self.h, int(which), roid, ne, corners.ctypes.data, u.ctypes.data, _p(uo), float(dt), int(ip_kind),
                                    nip if ip_kind == 2 else 0, _p(lips), val.ctypes.data, _p(der)))
        return val, der

    def set_mesh(self, roid, coords, conn):
        self.coords = np.ascontiguousarray(coords, np.float64)
        self.conn = np.ascontiguousarray(conn, np.int32)
        self.roid = roid
        self._c(self.lib.ora_set_mesh(self.h, roid, self.coords.shape[0], self.coords.ctypes.data, self.conn.shape[0], self.conn.ctypes.data))
        self.n_nodes = self.coords.shape[0]
        self.nnzb = self.lib.ora_nnz_blocks(self.h)
        self.b = DIM[roid] + 1

    def pattern(self):
        rp = np.empty(self.n_nodes + 1, np.int32)
        ci = np.empty(self.nnzb, np.int32)
        self._c(self.lib.ora_pattern(self.h, rp.ctypes.data, ci.ctypes.data))
        return rp, ci

    def coloring(self):
        c = np.empty(self.conn.shape[0], np.int32)
        self._c(self.lib.ora_coloring(self.h, c.ctypes.data))
        return c, self.lib.ora_num_colors(self.h)

    def set_dirichlet(self, dofs, vals):
        self.dofs = np.ascontiguousarray(dofs, np.int32)
        self.dvals = np.ascontiguousarray(vals, np.float64)
        self._c(self.lib.ora_set_dirichlet(self.h, self.dofs.size, self.dofs.ctypes.data, self.dvals.ctypes.data))

    def add_dirichlet(self, dofs, vals):
        r = np.ascontiguousarray(dofs, np.int32)
        v = np.ascontiguousarray(vals, np.float64)
        self._c(self.lib.ora_add_dirichlet(self.h, r.size, r.ctypes.data, v.ctypes.data))

    def add_wall(self, nodes):
        a = np.ascontiguousarray(nodes, np.int32)
        self._c(self.lib.ora_add_wall(self.h, a.size, a.ctypes.data))

    def add_inflow(self, vel, sides):
        v = np.ascontiguousarray(vel, np.float64).ravel()
        sd = np.ascontiguousarray(np.atleast_2d(sides), np.int32)
        self._c(self.lib.ora_add_inflow(self.h, sd.shape[0], sd.shape[1], sd.ctypes.data, v.ctypes.data))

    def assemble(self, U, U_old=None, dt=0.0, defect=True, jacobian=True, nthreads=1):
        U = np.ascontiguousarray(U, np.float64).ravel()
        uo = None if U_old is None else np.ascontiguousarray(U_old, np.float64).ravel()
        D = np.zeros(U.size) if defect else None
        J = np.zeros(self.nnzb * self.b * self.b) if jacobian else None
        self._c(self.lib.ora_assemble(self.h, U.ctypes.data, _p(uo), float(dt), _p(D), _p(J), int(nthreads)))
        return D, J

    def newton(self, U, U_old=None, dt=0.0, rtol=1e-8, maxit=100, lin_rtol=1e-4, lin_maxit=2000, ls_steps=6, nthreads=1):
        U = np.ascontiguousarray(U, np.float64).ravel().copy()
        uo = None if U_old is None else np.ascontiguousarray(U_old, np.float64).ravel()
        stats = np.zeros(5)
        self._c(self.lib.ora_newton(self.h, U.ctypes.data, _p(uo), float(dt), rtol, maxit, lin_rtol, lin_maxit, ls_steps,
                                    int(nthreads), stats.ctypes.data))
        return U, {"iterations": int(stats[0]), "linear_iterations": int(stats[1]), "rel_defect": stats[2],
                   "initial_defect": stats[3], "status": int(stats[4])}

    def bsr_mv(self, V, x):
        y = np.zeros_like(x)
        self._c(self.lib.ora_bsr_mv(self.h, np.ascontiguousarray(V).ctypes.data, np.ascontiguousarray(x).ctypes.data, y.ctypes.data))
        return y


def geometry(roid, corners):
    """FV1 geometry dump of one element: list of SCVF dicts + SCV volumes."""
    lib = load()
    nscvf = {2: 3, 3: 4, 4: 6, 6: 9, 8: 12}[roid]
    nsh = NSH[roid]
    out = np.zeros(nscvf * 40 + nsh)
    c = np.ascontiguousarray(corners, np.float64)
    if lib.ora_geometry(roid, c.ctypes.data, out.ctypes.data) != 0:
        raise RuntimeError("oracle geometry failed")
    scvf = []
    for i in range(nscvf):
        o = out[i * 40:(i + 1) * 40]
        scvf.append({"from": int(o[0]), "to": int(o[1]), "ip": o[2:5], "normal": o[5:8], "shape": o[8:8 + nsh],
                     "grad": o[16:40].reshape(8, 3)[:nsh]})
    return scvf, out[nscvf * 40:]


def ref_tables(roid):
    lib = load()
    nco, ne, ns = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    edges = np.zeros(24, np.int32); snc = np.zeros(6, np.int32); sides = np.zeros(24, np.int32); ef = np.zeros(24, np.int32)
    lib.ora_ref_tables(roid, ctypes.byref(nco), ctypes.byref(ne), edges.ctypes.data, ctypes.byref(ns), snc.ctypes.data,
                       sides.ctypes.data, ef.ctypes.data)
    return {"nco": nco.value, "edges": edges[:2 * ne.value].reshape(-1, 2), "sides": sides[:4 * ns.value].reshape(-1, 4),
            "side_nco": snc[:ns.value], "edge_face": ef[:2 * ne.value].reshape(-1, 2)}


# ---------------------------------------------------------------------------
# The reference's own element callbacks (oracle/_ref/libnsfv1_ref.so): the
# unmodified reference sources compiled against the ugcore stand-in in
# oracle/ugshim (make -C oracle ref). Only built where the reference checkout
# exists; used to pin this oracle.
# ---------------------------------------------------------------------------
REF_LIB = HERE / "_ref" / "libnsfv1_ref.so"
_ref_lib = None


class RefConfig(ctypes.Structure):
    _fields_ = [("nu", c_double), ("rho", c_double), ("full_newton", c_double), ("src", c_double * 3),
                ("has_source", c_int), ("stokes", c_int), ("laplace", c_int), ("peclet", c_int), ("pac", c_int),
                ("upwind", c_char_p), ("stab", c_char_p), ("diff_length", c_char_p), ("stab_upwind", c_char_p)]


def reference_root() -> Path | None:
    """The reference checkout (NSREF_ROOT, default /root/reference), or None."""
    root = Path(os.environ.get("NSREF_ROOT", "/root/reference"))
    return root if (root / "incompressible" / "fv1" / "navier_stokes_fv1.cpp").exists() else None


def build_ref(force: bool = False) -> Path | None:
    """Build oracle/_ref/libnsfv1_ref.so from the reference sources; None if they are absent."""
    root = reference_root()
    if root is None:
        return None
    subprocess.run(["make", "-C", str(HERE), "ref", f"NSREF_ROOT={root}"] + (["-B"] if force else []), check=True,
                   capture_output=True)
    return REF_LIB


def load_ref():
    global _ref_lib
    if _ref_lib is None:
        if build_ref() is None:
            raise RuntimeError("reference sources not available")
        lib = ctypes.CDLL(str(REF_LIB))
        lib.ref_elem_batch.restype = c_int
        lib.ref_elem_batch.argtypes = [c_int, c_int64, ctypes.POINTER(RefConfig), c_void_p, c_void_p, c_void_p, c_double,
                                       c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        lib.ref_geometry.restype = c_int
        lib.ref_geometry.argtypes = [c_int, c_void_p, c_void_p]
        lib.ref_outflow_batch.restype = c_int
        lib.ref_outflow_batch.argtypes = [c_int, c_int64, ctypes.POINTER(RefConfig), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        lib.ref_export.restype = c_int
        lib.ref_export.argtypes = [c_int, c_int, c_int64, ctypes.POINTER(RefConfig), c_void_p, c_void_p, c_void_p, c_double, c_int, c_int,
                                   c_void_p, c_void_p, c_void_p]
        lib.ref_last_error.restype = c_char_p
        _ref_lib = lib
    return _ref_lib


def _ref_cfg(cfg: dict):
    src = cfg.get("source")
    enc = lambda s: None if s is None else s.encode()
    return RefConfig(float(cfg.get("nu", 0.01)), float(cfg.get("rho", 1.0)), float(cfg.get("full_newton", 0.0)),
                     (c_double * 3)(*(list(src) + [0.0] * (3 - len(src)) if src is not None else [0.0, 0.0, 0.0])),
                     int(src is not None), int(bool(cfg.get("stokes"))), int(bool(cfg.get("laplace"))), int(bool(cfg.get("peclet"))),
                     int(bool(cfg.get("pac"))), enc(cfg["upwind"]), enc(cfg["stab"]), enc(cfg.get("diff_length")),
                     enc(cfg.get("stab_upwind")))


def ref_elem_batch(roid, cfg: dict, corners, u, u_old=None, dt=0.0, want=("defA", "jacA", "defM", "jacM", "rhs")):
    """The reference's add_*_elem outputs for n elements (same layouts as Oracle.elem_batch).
    cfg keys: nu, rho, full_newton, source (None or list), stokes, laplace, peclet, pac,
    upwind, stab, diff_length, stab_upwind."""
    lib = load_ref()
    corners = np.ascontiguousarray(corners, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    ne = corners.shape[0]
    nloc = (DIM[roid] + 1) * NSH[roid]
    out = {}
    for k in ("defA", "defM", "rhs"):
        out[k] = np.zeros((ne, nloc)) if k in want else None
    for k in ("jacA", "jacM"):
        out[k] = np.zeros((ne, nloc * nloc)) if k in want else None
    uo = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
    c = _ref_cfg(cfg)
    st = lib.ref_elem_batch(roid, ne, ctypes.byref(c), corners.ctypes.data, u.ctypes.data, _p(uo), float(dt), _p(out["defA"]),
                            _p(out["jacA"]), _p(out["defM"]), _p(out["jacM"]), _p(out["rhs"]))
    if st != 0:
        raise RuntimeError(f"reference error {st}: {lib.ref_last_error().decode()}")
    return {k: v for k, v in out.items() if v is not None}


# data exports of the disc (navier_stokes_fv1.cpp:894-1491), in the index order of ora_export / ref_export
EXPORTS = ("velocity", "velocity_grad", "velocity_ip", "pressure", "pressure_grad")
NSCVF = {2: 3, 3: 4, 4: 6, 6: 9, 8: 12}


def export_size(which, roid):
    dim = DIM[roid]
    return {0: dim, 1: dim * dim, 2: dim, 3: 1, 4: dim}[int(which)]


def export_nip(roid, ip_kind, local_ips=None):
    return NSCVF[roid] if ip_kind == 0 else NSH[roid] if ip_kind == 1 else int(np.asarray(local_ips).shape[0])


def ref_outflow(roid, cfg: dict, corners, u, side_mask):
    """The reference's NavierStokesNoNormalStressOutflowFV1 on n elements (layouts as
    Oracle.outflow_elem); side_mask[e] bit s marks reference side s as outflow boundary."""
    lib = load_ref()
    corners = np.ascontiguousarray(corners, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    m = np.ascontiguousarray(side_mask, np.uint32)
    ne, nl = corners.shape[0], (DIM[roid] + 1) * NSH[roid]
    d, J = np.zeros((ne, nl)), np.zeros((ne, nl * nl))
    c = _ref_cfg(cfg)
    st = lib.ref_outflow_batch(roid, ne, ctypes.byref(c), corners.ctypes.data, u.ctypes.data, m.ctypes.data, d.ctypes.data, J.ctypes.data)
    if st != 0:
        raise RuntimeError(f"reference error {st}: {lib.ref_last_error().decode()}")
    return d, J


def ref_export(which, roid, cfg: dict, corners, u, u_old=None, dt=0.0, ip_kind=0, local_ips=None, derivs=True):
    """The reference's own data export `which` of n elements (layouts as Oracle.export)."""
    lib = load_ref()
    corners = np.ascontiguousarray(corners, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    lips = None if local_ips is None else np.ascontiguousarray(local_ips, np.float64)
    ne, nip, vs, b = corners.shape[0], export_nip(roid, ip_kind, lips), export_size(which, roid), DIM[roid] + 1
    val = np.zeros((ne, nip, vs))
    der = np.zeros((ne, nip, b, NSH[roid], vs)) if derivs else None
    uo = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
    c = _ref_cfg(cfg)
    st = lib.ref_export(int(which), roid, ne, ctypes.byref(c), corners.ctypes.data, u.ctypes.data, _p(uo), float(dt), int(ip_kind),
                        nip if ip_kind == 2 else 0, _p(lips), val.ctypes.data, _p(der))
    if st != 0:
        raise RuntimeError(f"reference error {st}: {lib.ref_last_error().decode()}")
    return val, der


def ref_geometry(roid, corners):
    """The ugcore stand-in's FV1 geometry of one element (same layout as geometry())."""
    lib = load_ref()
    nscvf = {2: 3, 3: 4, 4: 6, 6: 9, 8: 12}[roid]
    nsh = NSH[roid]
    out = np.zeros(nscvf * 40 + nsh)
    c = np.ascontiguousarray(corners, np.float64)
    if lib.ref_geometry(roid, c.ctypes.data, out.ctypes.data) != 0:
        raise RuntimeError(lib.ref_last_error().decode())
    scvf = []
    for i in range(nscvf):
        o = out[i * 40:(i + 1) * 40]
        scvf.append({"from": int(o[0]), "to": int(o[1]), "ip": o[2:5], "normal": o[5:8], "shape": o[8:8 + nsh],
                     "grad": o[16:40].reshape(8, 3)[:nsh]})
    return scvf, out[nscvf * 40:]
