"""Python handle on the learned exit-direction surrogate (st_surrogate_* in
include/spacetime_gb300.h): FP64 GPU labels, BF16 tensor-core training with
AdamW, and inference."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

NIN, NOUT, NT = 6, 6, 8


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Surrogate:
    def __init__(self, device: int = 0, seed: int = 0):
        self._lib = _abi.load()
        h = C.c_void_p()
        _abi.check(self._lib.st_surrogate_create(C.byref(h), device, seed), "st_surrogate_create")
        self._h = h
        self.nparam = self._lib.st_surrogate_num_params()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.st_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        P = np.empty(self.nparam, np.float32)
        _abi.check(self._lib.st_surrogate_get_params(self._h, _fp(P)), "st_surrogate_get_params")
        return P

    def set_params(self, P):
        P = np.ascontiguousarray(P, dtype=np.float32)
        assert P.size == self.nparam
        _abi.check(self._lib.st_surrogate_set_params(self._h, _fp(P)), "st_surrogate_set_params")

    def forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.empty((X.shape[0], NOUT), np.float32)
        _abi.check(self._lib.st_surrogate_forward(self._h, _fp(X), X.shape[0], _fp(out)), "st_surrogate_forward")
        return out

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = np.empty(4, np.float32)
        g = np.empty(self.nparam, np.float32)
        _abi.check(self._lib.st_surrogate_loss_grad(self._h, _fp(X), _fp(T), X.shape[0], _fp(loss), _fp(g)),
                   "st_surrogate_loss_grad")
        return loss, g

    def generate(self, n: int, offset: int = 0, dt: float = 0.02, copy: bool = True):
        x = np.empty((n, NIN), np.float32) if copy else None
        t = np.empty((n, NT), np.float32) if copy else None
        raw = np.empty((n, 12), np.float32) if copy else None
        nul = C.POINTER(C.c_float)()
        _abi.check(self._lib.st_surrogate_generate(self._h, n, offset, dt, _fp(x) if copy else nul,
                                                   _fp(t) if copy else nul, _fp(raw) if copy else nul),
                   "st_surrogate_generate")
        return x, t, raw

    def train(self, steps: int, batch: int = 4096, lr: float = 1e-3, weight_decay: float = 1e-5) -> np.ndarray:
        hist = np.empty(steps, np.float32)
        _abi.check(self._lib.st_surrogate_train(self._h, steps, batch, lr, weight_decay, _fp(hist)),
                   "st_surrogate_train")
        return hist


def raw_to_geometry(raw):
    """(r, theta, a, n[3]) of label rows (raw[:, :6])."""
    return raw[:, 0], raw[:, 1], raw[:, 2], raw[:, 3:6]
