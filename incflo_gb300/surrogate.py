"""Learned warm start for the nodal solve: a 3-D U-Net trained on the GPU on pairs produced by this
library's own solver, evaluated on a coarse multigrid level of a nodal plan to supply the initial
guess of zero-guess projections (Galerkin-scaled, bypassed when not better than the zero start).

  s = Surrogate(seed=0)
  s.add_sample(projector)           # after projector.project(): rhs, sigma -> phi pair
  s.train(steps=600, lr=1e-3)       # Adam on the stored pairs (tensor-core forward / backward)
  projector.setSurrogate(s, level=1)
  projector.project()               # stats["warm_start"]: 1 used, 2 bypassed

No reference counterpart; everything runs in libincflo_gb300.so.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "unet16_seq128.bin")


def _ints(v):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Surrogate:
    def __init__(self, seed: int = 0, base: int = 16, path: str | None = None):
        self._L = A.load()
        p = ctypes.c_void_p()
        A.check(self._L.gbp_surrogate_create(base, seed, ctypes.byref(p)), "gbp_surrogate_create")
        self.ptr = p
        if path is not None:
            self.load(path)

    def __del__(self):
        if getattr(self, "ptr", None):
            self._L.gbp_surrogate_destroy(self.ptr)
            self.ptr = None

    @property
    def num_params(self) -> int:
        return int(self._L.gbp_surrogate_num_params(self.ptr))

    def params(self) -> np.ndarray:
        h = np.empty(self.num_params, dtype=np.float32)
        A.check(self._L.gbp_surrogate_get_params(self.ptr, h.ctypes.data, h.size), "gbp_surrogate_get_params")
        return h

    def set_params(self, h: np.ndarray):
        h = np.ascontiguousarray(h, dtype=np.float32)
        A.check(self._L.gbp_surrogate_set_params(self.ptr, h.ctypes.data, h.size), "gbp_surrogate_set_params")

    def grads(self) -> np.ndarray:
        h = np.empty(self.num_params, dtype=np.float32)
        A.check(self._L.gbp_surrogate_get_grads(self.ptr, h.ctypes.data, h.size), "gbp_surrogate_get_grads")
        return h

    def save(self, path: str):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        A.check(self._L.gbp_surrogate_save(self.ptr, path.encode()), "gbp_surrogate_save")

    def load(self, path: str):
        A.check(self._L.gbp_surrogate_load(self.ptr, path.encode()), "gbp_surrogate_load")

    def train_pair(self, x0: torch.Tensor, target: torch.Tensor, dims, dom, lr: float = 0.0) -> float:
        """One forward/backward (+ Adam step if lr > 0) on a device input [R, 16] bf16 and target [R] f32."""
        loss = ctypes.c_double()
        A.check(self._L.gbp_surrogate_train_pair(self.ptr, _ints(dims), _ints(dom), x0.data_ptr(), target.data_ptr(),
                                                 float(lr), ctypes.byref(loss), _stream()), "gbp_surrogate_train_pair")
        return loss.value

    def predict(self, x0: torch.Tensor, dims) -> torch.Tensor:
        rows = (dims[0] + 2) * (dims[1] + 2) * (dims[2] + 2)
        out = torch.empty((rows, 16), dtype=torch.bfloat16, device=x0.device)
        A.check(self._L.gbp_surrogate_predict(self.ptr, _ints(dims), x0.data_ptr(), out.data_ptr(), _stream()),
                "gbp_surrogate_predict")
        return out

    def add_sample(self, projector, phi_prev: torch.Tensor | None = None):
        """Store the (rhs, sigma[, phi_prev]) -> phi pair of a projector's last project() call."""
        from .projection import _ref, array4
        plan = projector._plan()
        pa = array4(phi_prev) if phi_prev is not None else None
        A.check(self._L.gbp_surrogate_add_sample(self.ptr, plan.ptr, _ref(pa)), "gbp_surrogate_add_sample")

    def train_step(self, projector, phi_prev: torch.Tensor | None = None, lr: float = 1e-3) -> float:
        """One Adam step on the (rhs, sigma, phi_prev) -> phi - phi_prev pair of a projector's (or a
        _Plan's) last projection, not stored; returns the loss."""
        from .projection import _ref, array4
        plan = projector._plan() if hasattr(projector, "_plan") else projector
        pa = array4(phi_prev) if phi_prev is not None else None
        loss = ctypes.c_double()
        A.check(self._L.gbp_surrogate_train_step(self.ptr, plan.ptr, _ref(pa), float(lr), ctypes.byref(loss)),
                "gbp_surrogate_train_step")
        return float(loss.value)

    @property
    def num_samples(self) -> int:
        return int(self._L.gbp_surrogate_num_samples(self.ptr))

    def clear_samples(self):
        A.check(self._L.gbp_surrogate_clear_samples(self.ptr), "gbp_surrogate_clear_samples")

    def train(self, steps: int, lr: float = 1e-3, seed: int = 0) -> list:
        """Adam steps on randomly drawn stored samples; returns the loss of every step."""
        out = []
        done = 0
        while done < steps:
            k = min(60, steps - done)
            buf = np.zeros(k, dtype=np.float32)
            A.check(self._L.gbp_surrogate_train(self.ptr, k, float(lr), seed * 1000003 + done, buf.ctypes.data,
                                                _stream()), "gbp_surrogate_train")
            out += buf.tolist()
            done += k
        return out
