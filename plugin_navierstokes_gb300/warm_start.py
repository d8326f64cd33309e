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
