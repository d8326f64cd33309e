"""Learned warm start of the batched cavity Newton solve.

``CoordinateMLP`` binds the tensor-core MLP of the native library
(nsfv1_mlp_*): a coordinate network (x, y) -> (u/lid, v/lid, p/lid^2),
FiLM-conditioned on (log Re, lid), trained with the library's own forward /
backward kernels and Adam, and used to write the Newton initial iterate of
every cavity instance. The plain FP64 defect judges the prediction: the batched
solver (``defect_reference="zero", zero_fallback=True``) restarts from the zero
iterate any instance whose predicted iterate has a larger defect than zero.
"""
from __future__ import annotations

import ctypes
import json
import os
from collections import Counter
from pathlib import Path

import numpy as np

from . import _capi
from ._capi import NSFV1Error


def condition(re: float, lid: float) -> np.ndarray:
    """Conditioning vector of one cavity (nsfv1_mlp_condition)."""
    c = np.zeros(2, np.float32)
    _capi.load().nsfv1_mlp_condition(float(re), float(lid), c.ctypes.data)
    return c


def _stream(stream):
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class CoordinateMLP:
    """Handle of one network (parameters, Adam state and staging buffers)."""

    def __init__(self, max_points: int = 65536, max_slots: int = 256, seed: int = 4):
        self._lib = _capi.load()
        self._h = ctypes.c_void_p()
        cfg = _capi.MlpConfig(int(max_points), int(max_slots))
        st = self._lib.nsfv1_mlp_create(ctypes.byref(cfg), ctypes.byref(self._h))
        if st != _capi.OK:
            raise NSFV1Error(st, "nsfv1_mlp_create failed")
        self.max_points, self.max_slots = int(max_points), int(max_slots)
        self.num_params = int(self._lib.nsfv1_mlp_num_params(self._h))
        self._check(self._lib.nsfv1_mlp_init(self._h, int(seed)))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.nsfv1_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def _check(self, st):
        if st != _capi.OK:
            raise NSFV1Error(st, self._lib.nsfv1_mlp_last_error(self._h).decode())

    # -- parameters ------------------------------------------------------------
    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, np.float32)
        self._check(self._lib.nsfv1_mlp_get_params(self._h, p.ctypes.data, self.num_params))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        self._check(self._lib.nsfv1_mlp_set_params(self._h, p.ctypes.data, p.size))

    # -- compute -----------------------------------------------------------------
    @staticmethod
    def _slots(slot_ptr):
        sp = np.ascontiguousarray(slot_ptr, np.int32)
        return sp, sp.size - 1

    def forward(self, xy, slot_ptr, cond, out, stream=None) -> None:
        """out[n, 3] (device FP32) = network output at xy[n, 2] (device FP32)."""
        sp, ns = self._slots(slot_ptr)
        c = np.ascontiguousarray(cond, np.float32)
        self._check(self._lib.nsfv1_mlp_forward(self._h, xy.shape[0], xy.data_ptr(), ns, sp.ctypes.data, c.ctypes.data,
                                                out.data_ptr(), _stream(stream)))

    def loss_grad(self, xy, slot_ptr, cond, target, grad, stream=None) -> float:
        """Loss and the gradient of every parameter (grad: device FP32 [num_params])."""
        sp, ns = self._slots(slot_ptr)
        c = np.ascontiguousarray(cond, np.float32)
        loss = ctypes.c_double()
        self._check(self._lib.nsfv1_mlp_loss_grad(self._h, xy.shape[0], xy.data_ptr(), ns, sp.ctypes.data, c.ctypes.data,
                                                  target.data_ptr(), ctypes.byref(loss), grad.data_ptr(), _stream(stream)))
        return loss.value

    def train(self, coords, targets, cond, steps: int, slots: int = 64, points_per_slot: int = 1024, lr: float = 2e-3,
              lr_final: float = 5e-5, seed: int = 4, step_offset: int = 0, record_loss: bool = True, stream=None):
        """Adam on minibatches of ``slots`` instances x ``points_per_slot`` nodes drawn
        on the device. coords [n_nodes, 2], targets [n_train, n_nodes, 3] and cond
        [n_train, 2] are device FP32 tensors. Returns the loss of every step."""
        ds = _capi.MlpDataset(targets.shape[0], coords.shape[0], coords.data_ptr(), targets.data_ptr(), cond.data_ptr())
        tp = _capi.MlpTrainParams(int(steps), int(slots), int(points_per_slot), float(lr), float(lr_final), int(seed), int(step_offset))
        hist = np.zeros(steps, np.float32) if record_loss else None
        self._check(self._lib.nsfv1_mlp_train(self._h, ctypes.byref(ds), ctypes.byref(tp),
                                              hist.ctypes.data if record_loss else None, _stream(stream)))
        return hist

    def predict(self, xy, slot_ptr, cond, lid, u, stream=None) -> None:
        """Writes the Newton initial iterate u[n*3] (device FP64) of every slot."""
        sp, ns = self._slots(slot_ptr)
        c = np.ascontiguousarray(cond, np.float32)
        l = np.ascontiguousarray(lid, np.float32)
        self._check(self._lib.nsfv1_mlp_predict(self._h, xy.shape[0], xy.data_ptr(), ns, sp.ctypes.data, c.ctypes.data, l.ctypes.data,
                                                u.data_ptr(), _stream(stream)))


def targets_from_solutions(u, lid, n_nodes: int, out, stream=None) -> None:
    """Normalised training targets (nsfv1_mlp_targets) of solutions that share one mesh."""
    n_inst = lid.shape[0]
    st = _capi.load().nsfv1_mlp_targets(n_inst, int(n_nodes), u.data_ptr(), lid.data_ptr(), out.data_ptr(), _stream(stream))
    if st != _capi.OK:
        raise NSFV1Error(st, "nsfv1_mlp_targets failed")


def gemm_bf16(A, B, splits: int = 1, stream=None):
    """C[splits, M, N] (FP32) = A[M, K] @ B[N, K]^T per K chunk on the tensor cores (nsfv1_gemm_bf16)."""
    import torch

    M, K = A.shape
    N = B.shape[0]
    lib = _capi.load()
    used = lib.nsfv1_gemm_bf16_splits(K, splits)
    if used <= 0:
        raise NSFV1Error(_capi.ERR_ARGUMENT, "K must be a positive multiple of 64")
    C = torch.empty((used, M, N), dtype=torch.float32, device=A.device)
    st = lib.nsfv1_gemm_bf16(M, N, K, A.data_ptr(), B.data_ptr(), C.data_ptr(), splits, _stream(stream))
    if st != _capi.OK:
        raise NSFV1Error(st, "nsfv1_gemm_bf16 failed")
    return C


# ---- batched cavities with a learned initial iterate -------------------------

class CavityBatch:
    """Independent lid-driven cavities (structured quads, full upwind + FLOW, as
    the batched workload) set up on one NavierStokesFV1 handle: per-element
    viscosity nu = lid / Re, instance ranges, multigrid hierarchy."""

    def __init__(self, N, Re, lid, upwind: str = "full", stabilization: str = "flow", exact_jacobian: float = 0.0):
        import torch

        from . import mesh
        from .navier_stokes_fv1 import NavierStokesFV1

        self.N = np.asarray(N, np.int32)
        self.Re = np.asarray(Re, np.float64)
        self.lid = np.asarray(lid, np.float64)
        B = mesh.cavity_batch(self.N, self.Re, self.lid)
        d = NavierStokesFV1("u,v,p", "Inner")
        d.set_kinematic_viscosity(1.0)
        d.set_upwind(upwind)
        d.set_stabilization(stabilization)
        d.set_exact_jacobian(exact_jacobian)
        d.set_mesh(B["elem_type"], B["coords"], B["conn"])
        d.set_elem_viscosity(B["nu_elem"])
        d.set_instances(B["node_offsets"])
        d.set_dirichlet(B["dofs"], B["values"])
        d.set_instance_grids(self.N)
        self.disc = d
        self.node_offsets = B["node_offsets"]
        self.n_nodes = int(B["coords"].shape[0])
        self.xy = torch.from_numpy(B["coords"].astype(np.float32)).cuda()
        self.cond = np.stack([condition(r, l) for r, l in zip(self.Re, self.lid)])
        self.exact_jacobian = float(exact_jacobian)
        self.cluster_size, self.smooth_steps, self.coarse_steps = 8, 2, 20

    def autotune(self, jacobian_prec: str = "f32", candidates=(4, 8, 16), smoothing=((2, 20), (3, 20), (2, 40), (3, 40)),
                 forcing_max: float = 0.0, cache_file: str | None = None) -> dict:
        """Picks the cluster size (CTAs per instance) and the V-cycle smoothing
        (pre/post sweeps, coarsest-level sweeps) of this batch by timing one
        Newton step per combination (nsfv1_batch_autotune per smoothing choice);
        the choice is cached in a JSON file keyed by device, precision, Newton
        options and the multiset of mesh sizes (default
        ~/.cache/nsfv1_gb300/autotune.json, or $NSFV1_AUTOTUNE_CACHE)."""
        import torch

        path = Path(cache_file or os.environ.get("NSFV1_AUTOTUNE_CACHE", Path.home() / ".cache" / "nsfv1_gb300" / "autotune.json"))
        key = "|".join([torch.cuda.get_device_name(), jacobian_prec, f"exact={self.exact_jacobian}", f"forcing={forcing_max}",
                        ",".join(map(str, candidates)), ",".join(f"{a}/{b}" for a, b in smoothing),
                        ",".join(f"{n}x{c}" for n, c in sorted(Counter(self.N.tolist()).items()))])
        cache = {}
        if path.exists():
            try:
                cache = json.loads(path.read_text())
            except (OSError, ValueError):
                cache = {}
        if key not in cache:
            u = self.zeros()
            trials = []
            for sm, co in smoothing:
                # timed with the fixed linear tolerance: a loose first adaptive step would hide the cost of later ones
                best, ms = self.disc.batch_autotune(u, candidates=candidates, jacobian_prec=jacobian_prec, smooth_steps=sm,
                                                    coarse_steps=co, forcing_max=0.0)
                trials.append((min(ms), best, sm, co))
            t, best, sm, co = min(trials)
            cache[key] = {"cluster_size": best, "smooth_steps": sm, "coarse_steps": co, "ms": t}
            try:
                path.parent.mkdir(parents=True, exist_ok=True)
                path.write_text(json.dumps(cache, indent=1))
            except OSError:
                pass
        c = cache[key]
        self.cluster_size, self.smooth_steps, self.coarse_steps = int(c["cluster_size"]), int(c["smooth_steps"]), int(c["coarse_steps"])
        return dict(c)

    @property
    def n_inst(self) -> int:
        return int(self.N.size)

    def zeros(self):
        import torch

        return torch.zeros(self.n_nodes * 3, dtype=torch.float64, device="cuda")

    def predict(self, model: "CoordinateMLP", u=None):
        """The network's initial iterate of every instance (FP64 device vector)."""
        u = self.zeros() if u is None else u
        model.predict(self.xy, self.node_offsets, self.cond, self.lid.astype(np.float32), u)
        return u

    def solve(self, u, jacobian_prec: str = "f32", rtol: float = 1e-8, defect_reference: str = "zero",
              zero_fallback: bool = False, **kw):
        """Batched Newton from u (in place); returns the per-instance results."""
        opts = dict(lin_rtol=1e-3, lin_max_iter=400, max_iter=80, cluster_size=self.cluster_size, smooth_steps=self.smooth_steps,
                    coarse_steps=self.coarse_steps, raise_on_error=False)
        opts.update(kw)
        return self.disc.newton_solve_batched(u, rtol=rtol, jacobian_prec=jacobian_prec, defect_reference=defect_reference,
                                              zero_fallback=zero_fallback, **opts)


def generate_training_set(Re, lid, N: int = 128, batch: int = 256, jacobian_prec: str = "f32", **solve_kw):
    """Solves cavities of one mesh size (N x N cells) in batches with the batched
    Newton and returns (coords [n_nodes, 2], targets [n, n_nodes, 3], cond [n, 2],
    results) on the device, targets normalised as nsfv1_mlp_targets."""
    import torch

    Re = np.asarray(Re, np.float64)
    lid = np.asarray(lid, np.float64)
    n = Re.size
    nn = (N + 1) ** 2
    targets = torch.empty((n, nn, 3), dtype=torch.float32, device="cuda")
    results = []
    coords = None
    for s in range(0, n, batch):
        e = min(n, s + batch)
        cb = CavityBatch(np.full(e - s, N), Re[s:e], lid[s:e])
        u = cb.zeros()
        results += cb.solve(u, jacobian_prec=jacobian_prec, **solve_kw)
        lt = torch.from_numpy(lid[s:e]).cuda()
        targets_from_solutions(u, lt, nn, targets[s:e])
        if coords is None:
            coords = cb.xy[:nn].clone()
        del cb
    cond = torch.from_numpy(np.stack([condition(r, l) for r, l in zip(Re, lid)])).cuda()
    torch.cuda.synchronize()
    return coords, targets, cond, results
