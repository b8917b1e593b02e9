"""Python handle on the learned exit-direction surrogate (st_surrogate_* in
include/spacetime_gb300.h): FP64 GPU labels, BF16 tensor-core training with
AdamW, and inference."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi

NIN, NOUT, NT = 6, 6, 8
RAW = 15  # label row: r, theta, a, n (3), flags, steps, exit dir (3), r_cross, launch dir d0 (3)


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

    def forward_tc(self, X) -> np.ndarray:
        """The network on the frame pass's tcgen05 / TMEM kernel."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.empty((X.shape[0], NOUT), np.float32)
        _abi.check(self._lib.st_surrogate_forward_tc(self._h, _fp(X), X.shape[0], _fp(out)),
                   "st_surrogate_forward_tc")
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
        raw = np.empty((n, RAW), np.float32) if copy else None
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


TRAINED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "surrogate_kerr.npy")


def load_trained(device: int = 0) -> "Surrogate":
    """The shipped network (spacetime_gb300/data/surrogate_kerr.npy, made by
    spacetime_gb300/train_surrogate.py)."""
    s = Surrogate(device)
    s.set_params(np.load(TRAINED))
    return s


def raw_to_geometry(raw):
    """(r, theta, a, n[3]) of label rows (raw[:, :6])."""
    return raw[:, 0], raw[:, 1], raw[:, 2], raw[:, 3:6]


def label_position_unit(raw):
    """Unit Cartesian position of each label row's camera, at azimuth 0:
    pos = (sqrt(r^2 + a^2) sin theta, 0, r cos theta)."""
    r, th, a = (raw[:, k].astype(np.float64) for k in range(3))
    pos = np.stack([np.sqrt(r * r + a * a) * np.sin(th), np.zeros_like(r), r * np.cos(th)], 1)
    return pos / np.linalg.norm(pos, axis=1, keepdims=True)


def plane_exit(xh, d0, defl, tilt):
    """Exit direction from the network's ray-plane angles (the gate's
    reconstruction): cos E (cos(psi + D) xh + sin(psi + D) et) + sin E en."""
    xh = np.asarray(xh, np.float64)
    d0 = np.asarray(d0, np.float64)
    d0 = d0 / np.linalg.norm(d0, axis=1, keepdims=True)
    c = (xh * d0).sum(1)
    t = d0 - c[:, None] * xh
    sn = np.linalg.norm(t, axis=1)
    et = t / np.maximum(sn, 1e-300)[:, None]
    en = np.cross(xh, et)
    psi = np.arctan2(sn, c)
    chi = psi + np.asarray(defl, np.float64)
    e = np.asarray(tilt, np.float64)[:, None]
    d = np.cos(e) * (np.cos(chi)[:, None] * xh + np.sin(chi)[:, None] * et) + np.sin(e) * en
    return d / np.linalg.norm(d, axis=1, keepdims=True)
