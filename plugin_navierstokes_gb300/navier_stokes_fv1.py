"""Host-side mirror of the reference's ``NavierStokesFV1`` element disc.

Same method names, string ids, defaults and error behaviour as the reference
(incompressible/fv1/navier_stokes_fv1.h:160-225, navier_stokes_base.h:163-196,
incompressible_navier_stokes_base.h:183-225, registered for Lua in
incompressible/fv1/register_fv1.cpp:167-184); every call goes through the
C ABI of ``libnsfv1_gb300.so``. Device vectors are torch CUDA tensors (torch is
only the device-memory / stream plumbing here).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import NSFV1Error, check


def _ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class NavierStokesFV1:
    """``NavierStokesFV1(fcts, subsets)`` (navier_stokes_fv1.cpp:45-87) for dim 2 or 3.

    ``functions``/``subsets`` are accepted for API parity; the disc always
    carries dim+1 P1 functions (u, v, [w], p) like the reference's init check.
    """

    def __init__(self, functions: str | list[str] = "", subsets: str | list[str] = "", dim: int | None = None):
        fcts = [f.strip() for f in functions.split(",")] if isinstance(functions, str) else list(functions)
        fcts = [f for f in fcts if f]
        if dim is None:
            dim = len(fcts) - 1 if fcts else 2
        if fcts and len(fcts) != dim + 1:
            raise NSFV1Error(_capi.ERR_ARGUMENT, f"Wrong number of functions: The ElemDisc 'NavierStokes' needs exactly {dim + 1} symbolic function.")
        self.dim = dim
        self.functions = fcts
        self.subsets = subsets
        self._lib = _capi.load()
        h = ctypes.c_void_p()
        st = self._lib.nsfv1_create(dim, ctypes.byref(h))
        if st != _capi.OK:
            raise NSFV1Error(st, "nsfv1_create failed")
        self._h = h
        self.elem_type = None
        self.n_nodes = 0
        self.n_elems = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.nsfv1_destroy(h)
            self._h = None

    def _c(self, st: int) -> None:
        check(self._h, st)

    # ---- reference setters -------------------------------------------------
    def disc_type(self) -> str:
        return self._lib.nsfv1_disc_type(self._h).decode()

    def set_kinematic_viscosity(self, nu: float) -> None:
        self._c(self._lib.nsfv1_set_kinematic_viscosity(self._h, float(nu)))

    def set_density(self, rho: float) -> None:
        self._c(self._lib.nsfv1_set_density(self._h, float(rho)))

    def set_source(self, f) -> None:
        a = np.ascontiguousarray(np.asarray(f, dtype=np.float64))
        self._c(self._lib.nsfv1_set_source(self._h, a.ctypes.data, a.size))

    def set_exact_jacobian(self, v) -> None:
        factor = (1.0 if v else 0.0) if isinstance(v, bool) else float(v)
        self._c(self._lib.nsfv1_set_exact_jacobian(self._h, factor))

    def set_stokes(self, on: bool) -> None:
        self._c(self._lib.nsfv1_set_stokes(self._h, int(bool(on))))

    def set_laplace(self, on: bool) -> None:
        self._c(self._lib.nsfv1_set_laplace(self._h, int(bool(on))))

    def set_peclet_blend(self, on: bool) -> None:
        self._c(self._lib.nsfv1_set_peclet_blend(self._h, int(bool(on))))

    def set_upwind(self, name: str) -> None:
        self._c(self._lib.nsfv1_set_upwind(self._h, name.encode()))

    def set_stabilization(self, name: str, diff_length: str | None = None) -> None:
        self._c(self._lib.nsfv1_set_stabilization(self._h, name.encode(), diff_length.encode() if diff_length else None))

    def set_pac_upwind(self, on: bool) -> None:
        """set_pac_upwind (navier_stokes_fv1.h:217-225): the stabilised velocity as the convective upwind."""
        self._c(self._lib.nsfv1_set_pac_upwind(self._h, int(bool(on))))

    def set_stabilization_upwind(self, name: str) -> None:
        self._c(self._lib.nsfv1_set_stabilization_upwind(self._h, name.encode()))

    # ---- mesh ----------------------------------------------------------------
    def set_mesh(self, elem_type: int, coords: np.ndarray, conn: np.ndarray) -> None:
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        n_nodes = coords.shape[0]
        n_elems = conn.shape[0]
        self._c(self._lib.nsfv1_set_mesh(self._h, int(elem_type), n_nodes, coords.ctypes.data, n_elems, conn.ctypes.data))
        self.elem_type = elem_type
        self.n_nodes = n_nodes
        self.n_elems = n_elems

    def pattern_info(self) -> dict:
        nr, nnz = ctypes.c_int64(), ctypes.c_int64()
        bs, nc = ctypes.c_int(), ctypes.c_int()
        self._c(self._lib.nsfv1_pattern_info(self._h, ctypes.byref(nr), ctypes.byref(nnz), ctypes.byref(bs), ctypes.byref(nc)))
        return {"n_rows": nr.value, "nnz_blocks": nnz.value, "block_size": bs.value, "n_colors": nc.value}

    def pattern(self) -> tuple[np.ndarray, np.ndarray]:
        info = self.pattern_info()
        rp = np.empty(info["n_rows"] + 1, np.int32)
        ci = np.empty(info["nnz_blocks"], np.int32)
        self._c(self._lib.nsfv1_get_pattern(self._h, rp.ctypes.data, ci.ctypes.data))
        return rp, ci

    def coloring(self) -> np.ndarray:
        c = np.empty(self.n_elems, np.int32)
        self._c(self._lib.nsfv1_get_coloring(self._h, c.ctypes.data))
        return c

    def set_dirichlet(self, dofs: np.ndarray, values: np.ndarray) -> None:
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        values = np.ascontiguousarray(values, dtype=np.float64)
        self._c(self._lib.nsfv1_set_dirichlet(self._h, dofs.size, dofs.ctypes.data, values.ctypes.data))

    def add_dirichlet(self, dofs, values) -> None:
        """Appends Dirichlet rows (later values of the same unknown win; nsfv1_add_dirichlet)."""
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        values = np.ascontiguousarray(values, dtype=np.float64)
        self._c(self._lib.nsfv1_add_dirichlet(self._h, dofs.size, dofs.ctypes.data, values.ctypes.data))

    def clear_boundary(self) -> None:
        """Removes every Dirichlet row and inflow flux (nsfv1_clear_boundary)."""
        self._c(self._lib.nsfv1_clear_boundary(self._h))

    # ---- assembly (torch CUDA tensors) ----------------------------------------
    def assemble_defect(self, u, d, u_old=None, dt: float = 0.0, stream=None) -> None:
        self._c(self._lib.nsfv1_assemble_defect(self._h, _ptr(u), _ptr(u_old), float(dt), _ptr(d), _stream_ptr(stream)))

    def assemble_jacobian(self, u, vals, u_old=None, dt: float = 0.0, stream=None) -> None:
        import torch

        prec = _capi.F64 if vals.dtype == torch.float64 else _capi.F32
        self._c(self._lib.nsfv1_assemble_jacobian(self._h, _ptr(u), _ptr(u_old), float(dt), _ptr(vals), prec, _stream_ptr(stream)))

    def assemble_defect_jacobian(self, u, d, vals, u_old=None, dt: float = 0.0, stream=None) -> None:
        """Defect into d and Jacobian into vals at the same u, in one pass over the elements."""
        import torch

        prec = _capi.F64 if vals.dtype == torch.float64 else _capi.F32
        self._c(self._lib.nsfv1_assemble_defect_jacobian(self._h, _ptr(u), _ptr(u_old), float(dt), _ptr(d), _ptr(vals), prec,
                                                         _stream_ptr(stream)))

    def elem_batch(self, elem_type: int, corners, u, u_old=None, dt: float = 0.0, defA=None, jacA=None, defM=None,
                   jacM=None, rhs=None, stream=None) -> None:
        n = corners.shape[0]
        self._c(self._lib.nsfv1_elem_batch(self._h, int(elem_type), n, _ptr(corners), _ptr(u), _ptr(u_old), float(dt),
                                           _ptr(defA), _ptr(jacA), _ptr(defM), _ptr(jacM), _ptr(rhs), _stream_ptr(stream)))

    # ---- post-processing (navier_stokes_tools.h) ----
    def vorticity(self, u, vort, stream=None) -> None:
        """vorticityFV1: the SCV-averaged corner curl of the P1 velocity, one value per node."""
        self._c(self._lib.nsfv1_vorticity(self._h, _ptr(u), _ptr(vort), _stream_ptr(stream)))

    def eval_points(self, u, points, fct: int, stream=None):
        """Function fct (0..dim) of the P1 solution u at global points [n][dim] (device tensor);
        returns a device tensor of n values, NaN outside the mesh."""
        import torch

        pts = points.contiguous()
        out = torch.empty(pts.shape[0], dtype=torch.float64, device=pts.device)
        self._c(self._lib.nsfv1_eval_points(self._h, _ptr(u), pts.shape[0], _ptr(pts), int(fct), _ptr(out), _stream_ptr(stream)))
        return out

    # ---- data exports (navier_stokes_fv1.cpp:894-1491; the accessors of
    # incompressible_navier_stokes_base.h:237-249) ----
    def velocity(self) -> "DataExport":
        return DataExport(self, EX_VELOCITY)

    def velocity_grad(self) -> "DataExport":
        return DataExport(self, EX_VELOCITY_GRAD)

    def velocity_ip(self) -> "DataExport":
        return DataExport(self, EX_VELOCITY_IP)

    def pressure(self) -> "DataExport":
        return DataExport(self, EX_PRESSURE)

    def pressure_grad(self) -> "DataExport":
        return DataExport(self, EX_PRESSURE_GRAD)

    def export(self, which: int, elem_type: int, corners, u, values, u_old=None, dt: float = 0.0, points="scvf", derivs=None,
               stream=None) -> None:
        """Export `which` of n elements into device arrays values [n][nip][vs] and, if given,
        derivs [n][nip][dim+1][corners][vs]; points "scvf", "scv" or a local-point array [nip][dim]."""
        if isinstance(points, str):
            kind, nip, lips = {"scvf": 0, "scv": 1}[points], 0, None
        else:
            lips = np.ascontiguousarray(points, np.float64)
            kind, nip = 2, int(lips.shape[0])
        n = corners.shape[0]
        self._c(self._lib.nsfv1_export(self._h, int(which), int(elem_type), n, _ptr(corners), _ptr(u), _ptr(u_old), float(dt), kind,
                                       nip, None if lips is None else lips.ctypes.data, _ptr(values), _ptr(derivs),
                                       _stream_ptr(stream)))

    def bsr_mv(self, vals, x, y, stream=None) -> None:
        import torch

        prec = _capi.F64 if vals.dtype == torch.float64 else _capi.F32
        self._c(self._lib.nsfv1_bsr_mv(self._h, _ptr(vals), prec, _ptr(x), _ptr(y), _stream_ptr(stream)))

    def split_vector(self, x, xs=None, stream=None):
        """x (FP64, device) as float pairs (xs: float32 of twice the length), the operand of bsr_mv_split."""
        import torch

        if xs is None:
            xs = torch.empty(2 * x.numel(), dtype=torch.float32, device=x.device)
        st = self._lib.nsfv1_split_vector(int(x.numel()), _ptr(x), _ptr(xs), _stream_ptr(stream))
        if st != 0:
            raise _capi.NSFV1Error(st, "split_vector failed")
        return xs

    def bsr_mv_split(self, vals, xs, y, stream=None) -> None:
        """y = J x for FP32 values and x split by split_vector (the BiCGStab loop's SpMV)."""
        self._c(self._lib.nsfv1_bsr_mv_split(self._h, _ptr(vals), _ptr(xs), _ptr(y), _stream_ptr(stream)))

    def block_jacobi(self, vals, r, z, stream=None) -> None:
        """z = D^-1 r with D the block diagonal of the Jacobian vals."""
        import torch

        prec = _capi.F64 if vals.dtype == torch.float64 else _capi.F32
        self._c(self._lib.nsfv1_block_jacobi(self._h, _ptr(vals), prec, _ptr(r), _ptr(z), _stream_ptr(stream)))

    def newton_solve(self, u, u_old=None, dt: float = 0.0, rtol: float = 1e-8, atol: float = 0.0, max_iter: int = 100,
                     lin_rtol: float = 1e-4, lin_max_iter: int = 2000, line_search_steps: int = 6, jacobian_prec: str = "f64",
                     linear_solver: str = "bicgstab", gmres_restart: int = 30, stream=None, raise_on_error: bool = True) -> dict:
        p = _capi.NewtonParams(rtol, atol, max_iter, lin_rtol, lin_max_iter, line_search_steps,
                               _capi.F64 if jacobian_prec == "f64" else _capi.F32,
                               _capi.GMRES if linear_solver == "gmres" else _capi.BICGSTAB, gmres_restart)
        r = _capi.NewtonResult()
        st = self._lib.nsfv1_newton_solve(self._h, _ptr(u), _ptr(u_old), float(dt), ctypes.byref(p), ctypes.byref(r),
                                          _stream_ptr(stream))
        res = {"status": r.status, "iterations": r.iterations, "linear_iterations": r.linear_iterations,
               "initial_defect": r.initial_defect, "final_defect": r.final_defect}
        if st != _capi.OK and raise_on_error:
            raise NSFV1Error(st, self._lib.nsfv1_last_error(self._h).decode() + f" {res}")
        return res

    def linear_solve(self, vals, rhs, x, lin_rtol: float = 1e-4, lin_max_iter: int = 2000, linear_solver: str = "bicgstab",
                     gmres_restart: int = 30, stream=None, raise_on_error: bool = True) -> dict:
        """J x = rhs with the Newton loop's linear solver (nsfv1_linear_solve); the
        precision of J follows vals' dtype. Returns status, iterations, relres, restarts."""
        import torch

        p = _capi.NewtonParams(0.0, 0.0, 1, lin_rtol, lin_max_iter, 0,
                               _capi.F64 if vals.dtype == torch.float64 else _capi.F32,
                               _capi.GMRES if linear_solver == "gmres" else _capi.BICGSTAB, gmres_restart)
        it, rr, rs = ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_int(0)
        st = self._lib.nsfv1_linear_solve(self._h, _ptr(vals), _ptr(rhs), _ptr(x), ctypes.byref(p), ctypes.byref(it),
                                          ctypes.byref(rr), ctypes.byref(rs), _stream_ptr(stream))
        res = {"status": st, "iterations": it.value, "relres": rr.value, "restarts": rs.value}
        if st != _capi.OK and raise_on_error:
            raise NSFV1Error(st, self._lib.nsfv1_last_error(self._h).decode() + f" {res}")
        return res

    def set_elem_viscosity(self, nu) -> None:
        """Per-element kinematic viscosity (None: back to the constant)."""
        if nu is None:
            self._c(self._lib.nsfv1_set_elem_viscosity(self._h, None))
            return
        a = np.ascontiguousarray(nu, dtype=np.float64)
        self._c(self._lib.nsfv1_set_elem_viscosity(self._h, a.ctypes.data))

    def set_instances(self, node_offsets) -> None:
        a = np.ascontiguousarray(node_offsets, dtype=np.int32)
        self._c(self._lib.nsfv1_set_instances(self._h, a.size - 1, a.ctypes.data))
        self.n_inst = a.size - 1

    def set_instance_grids(self, cells) -> None:
        """Structured square instances (cells per side) -> multigrid hierarchy."""
        a = np.ascontiguousarray(cells, dtype=np.int32)
        self._c(self._lib.nsfv1_set_instance_grids(self._h, a.ctypes.data))

    def newton_solve_batched(self, u, u_old=None, dt: float = 0.0, rtol: float = 1e-8, atol: float = 0.0, max_iter: int = 100,
                             lin_rtol: float = 1e-3, lin_max_iter: int = 3000, line_search_steps: int = 6,
                             jacobian_prec: str = "f64", gmres_restart: int = 30, cluster_size: int = 4, max_clusters: int = 0,
                             multigrid: bool = True, smooth_steps: int = 2, coarse_steps: int = 20, smooth_omega: float = 0.7,
                             defect_reference: str = "initial", zero_fallback: bool = False, forcing_max: float = 0.0,
                             graph: bool = True, tail_clusters: bool = True, stream=None, raise_on_error: bool = True) -> list[dict]:
        """Newton on every instance (nsfv1_newton_solve_batched). ``defect_reference``
        "initial" measures rtol against each instance's own initial defect, "zero"
        against the defect of the zero iterate; with "zero", ``zero_fallback``
        restarts from the zero iterate every instance whose given iterate has the
        larger defect. ``forcing_max`` > 0 switches on Eisenstat-Walker linear
        tolerances in [lin_rtol, forcing_max]; ``graph`` replays each step's fixed
        device work as one captured CUDA graph (one per cluster size); ``tail_clusters``
        grows the clusters of the remaining instances once few are active."""
        if defect_reference not in ("initial", "zero"):
            raise NSFV1Error(_capi.ERR_ARGUMENT, f"unknown defect reference '{defect_reference}'")
        p = _capi.NewtonParams(rtol, atol, max_iter, lin_rtol, lin_max_iter, line_search_steps,
                               _capi.F64 if jacobian_prec == "f64" else _capi.F32, _capi.GMRES, gmres_restart)
        o = _capi.BatchOptions(cluster_size, max_clusters, 1 if multigrid else 0, smooth_steps, coarse_steps, smooth_omega,
                               1 if defect_reference == "zero" else 0, 1 if zero_fallback else 0, float(forcing_max),
                               1 if graph else 0, 1 if tail_clusters else 0)
        res = (_capi.NewtonResult * self.n_inst)()
        st = self._lib.nsfv1_newton_solve_batched(self._h, _ptr(u), _ptr(u_old), float(dt), ctypes.byref(p), ctypes.byref(o),
                                                  ctypes.addressof(res), _stream_ptr(stream))
        out = [{"status": r.status, "iterations": r.iterations, "linear_iterations": r.linear_iterations,
                "initial_defect": r.initial_defect, "final_defect": r.final_defect} for r in res]
        if st not in (_capi.OK,) and raise_on_error:
            raise NSFV1Error(st, self._lib.nsfv1_last_error(self._h).decode())
        return out

    def batch_stats(self) -> dict:
        """Timing of the last batched solve (nsfv1_batch_stats)."""
        out = np.zeros(8)
        self._c(self._lib.nsfv1_batch_stats(self._h, out.ctypes.data, 8))
        return {"steps": int(out[0]), "step_work_ms": out[1], "line_search_ms": out[2], "wall_ms": out[3]}

    def set_assembly_threads(self, threads: int) -> None:
        """CTA size of the assembly colour launches (32, 64, 96 or 128)."""
        self._c(self._lib.nsfv1_set_assembly_threads(self._h, int(threads)))

    def assembly_threads(self) -> int:
        return int(self._lib.nsfv1_get_assembly_threads(self._h))

    def assembly_autotune(self, u, jacobian_prec: str = "f64", candidates=(32, 64, 128), stream=None) -> tuple[int, list[float]]:
        """Times defect + Jacobian assembly at u per CTA size (nsfv1_assembly_autotune) and
        keeps the fastest; returns (CTA size, milliseconds per candidate)."""
        c = np.ascontiguousarray(candidates, dtype=np.int32)
        ms = np.zeros(c.size)
        self._c(self._lib.nsfv1_assembly_autotune(self._h, _ptr(u), _capi.F64 if jacobian_prec == "f64" else _capi.F32,
                                                  c.ctypes.data, c.size, ms.ctypes.data, _stream_ptr(stream)))
        return self.assembly_threads(), [float(x) for x in ms]

    def batch_autotune(self, u, u_old=None, dt: float = 0.0, candidates=(2, 4, 8, 16), jacobian_prec: str = "f32",
                       lin_rtol: float = 1e-3, lin_max_iter: int = 400, gmres_restart: int = 30, multigrid: bool = True,
                       smooth_steps: int = 2, coarse_steps: int = 20, smooth_omega: float = 0.7,
                       forcing_max: float = 0.0, graph: bool = True, stream=None) -> tuple[int, list[float]]:
        """Times one batched Newton step per candidate cluster size (nsfv1_batch_autotune);
        returns (fastest cluster size, milliseconds per candidate). u is not changed."""
        p = _capi.NewtonParams(1e-8, 0.0, 1, lin_rtol, lin_max_iter, 6, _capi.F64 if jacobian_prec == "f64" else _capi.F32,
                               _capi.GMRES, gmres_restart)
        o = _capi.BatchOptions(0, 0, 1 if multigrid else 0, smooth_steps, coarse_steps, smooth_omega, 0, 0, float(forcing_max),
                               1 if graph else 0, 0)
        c = np.ascontiguousarray(candidates, dtype=np.int32)
        ms = np.zeros(c.size)
        self._c(self._lib.nsfv1_batch_autotune(self._h, _ptr(u), _ptr(u_old), float(dt), ctypes.byref(p), ctypes.byref(o),
                                               c.ctypes.data, c.size, ms.ctypes.data, _stream_ptr(stream)))
        return int(o.cluster_size), [float(x) for x in ms]

    def last_error(self) -> str:
        return self._lib.nsfv1_last_error(self._h).decode()


def mesh_pattern(elem_type: int, n_nodes: int, conn: np.ndarray):
    """Host-only block-CSR pattern + greedy colouring (nsfv1_mesh_pattern)."""
    lib = _capi.load()
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nnz, nc = ctypes.c_int64(), ctypes.c_int()
    st = lib.nsfv1_mesh_pattern(int(elem_type), n_nodes, conn.shape[0], conn.ctypes.data, ctypes.byref(nnz), ctypes.byref(nc), None, None, None)
    if st != _capi.OK:
        raise NSFV1Error(st, "nsfv1_mesh_pattern failed")
    rp = np.empty(n_nodes + 1, np.int32)
    ci = np.empty(nnz.value, np.int32)
    col = np.empty(conn.shape[0], np.int32)
    st = lib.nsfv1_mesh_pattern(int(elem_type), n_nodes, conn.shape[0], conn.ctypes.data, ctypes.byref(nnz), ctypes.byref(nc),
                                rp.ctypes.data, ci.ctypes.data, col.ctypes.data)
    if st != _capi.OK:
        raise NSFV1Error(st, "nsfv1_mesh_pattern failed")
    return rp, ci, col, nc.value


EX_VELOCITY, EX_VELOCITY_GRAD, EX_VELOCITY_IP, EX_PRESSURE, EX_PRESSURE_GRAD = range(5)
_NSCVF = {2: 3, 3: 4, 4: 6, 6: 9, 8: 12}
_NSH = {2: 3, 3: 4, 4: 4, 6: 6, 8: 8}


class DataExport:
    """One of the disc's data exports (the reference's velocity(), velocity_grad(),
    velocity_ip(), pressure(), pressure_grad() return a CplUserData that ugcore
    evaluates per element at integration points): evaluate() runs it on the GPU for
    a batch of elements and returns torch tensors (values, derivatives or None)."""

    def __init__(self, disc: NavierStokesFV1, which: int):
        self.disc, self.which = disc, which

    def value_size(self) -> int:
        dim = self.disc.dim
        return {EX_VELOCITY: dim, EX_VELOCITY_GRAD: dim * dim, EX_VELOCITY_IP: dim, EX_PRESSURE: 1, EX_PRESSURE_GRAD: dim}[self.which]

    def evaluate(self, elem_type: int, corners, u, u_old=None, dt: float = 0.0, points="scvf", derivs: bool = False, stream=None):
        import torch

        n = corners.shape[0]
        if isinstance(points, str):
            nip = {"scvf": _NSCVF[elem_type], "scv": _NSH[elem_type]}[points]
        else:
            nip = int(np.asarray(points).shape[0])
        vs = self.value_size()
        vals = torch.empty((n, nip, vs), dtype=torch.float64, device=corners.device)
        der = torch.empty((n, nip, self.disc.dim + 1, _NSH[elem_type], vs), dtype=torch.float64, device=corners.device) if derivs else None
        self.disc.export(self.which, elem_type, corners, u, vals, u_old, dt, points, der, stream)
        return vals, der


class NavierStokesWall:
    """``NavierStokesWall(master)`` (incompressible/bnd/wall.h, wall_impl.h:44-69):
    ``add(nodes)`` makes every velocity component of the nodes a zero Dirichlet row.
    The reference's ``add(subsets)`` takes subset names of ugcore's grid; here the
    caller passes the node ids of those subsets (nsfv1_add_wall)."""

    def __init__(self, master: NavierStokesFV1):
        self.master = master

    def add(self, nodes) -> None:
        a = np.ascontiguousarray(nodes, dtype=np.int32)
        self.master._c(self.master._lib.nsfv1_add_wall(self.master._h, a.size, a.ctypes.data))


class NavierStokesInflowFV1:
    """``NavierStokesInflowFV1(master)`` (incompressible/fv1/bnd/inflow_fv1.h,
    inflow_fv1_impl.h:42-82): ``add(velocity, sides)`` sets Dirichlet velocity rows
    on the nodes of the boundary sides and the continuity equation's Neumann flux
    vel . n over each corner's part of the sides (nsfv1_add_inflow). ``sides`` is
    an (n_sides, nodes per side) array of node ids (edges in 2D; triangles or
    quadrilaterals in 3D) standing for the reference's boundary subset names."""

    def __init__(self, master: NavierStokesFV1):
        self.master = master

    def add(self, velocity, sides) -> None:
        v = np.ascontiguousarray(np.asarray(velocity, dtype=np.float64).ravel())
        sd = np.ascontiguousarray(np.atleast_2d(np.asarray(sides, dtype=np.int32)))
        if v.size != self.master.dim:
            raise NSFV1Error(_capi.ERR_ARGUMENT, "NavierStokesInflow::add: the velocity needs dim components")
        self.master._c(self.master._lib.nsfv1_add_inflow(self.master._h, sd.shape[0], sd.shape[1], sd.ctypes.data, v.ctypes.data))


class NavierStokesNoNormalStressOutflowFV1:
    """``NavierStokesNoNormalStressOutflowFV1(master)`` (incompressible/fv1/bnd/
    no_normal_stress_outflow_fv1.cpp:343-504): ``add(sides)`` makes the given
    boundary sides an outflow boundary without normal stress -- the tangential
    viscous flux, the outgoing convective flux and the continuity flux of each
    corner's boundary face enter the defect and the Jacobian (nsfv1_add_outflow).
    ``sides`` is an (n_sides, nodes per side) array of node ids standing for the
    reference's boundary subset names."""

    def __init__(self, master: NavierStokesFV1):
        self.master = master

    def add(self, sides) -> None:
        sd = np.ascontiguousarray(np.atleast_2d(np.asarray(sides, dtype=np.int32)))
        self.master._c(self.master._lib.nsfv1_add_outflow(self.master._h, sd.shape[0], sd.shape[1], sd.ctypes.data))
