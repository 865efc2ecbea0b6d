"""Learned warm start of the Johnson-Cook return mapping (host side).

``Mlp`` owns an ``sph_mlp`` (include/sphfem.h): a 4-64-64-64-1 SiLU network
with BF16 weights whose layers, gradients and Adam updates run in the sm_103a
library (tensor-core tiles).  ``features`` turns the return-mapping records a
context logs (``Solver.jc_log_read``) into the network's inputs and target;
the device computes the same inputs for every yielding particle when the
network is attached (``Solver.attach_mlp``), and the secant return mapping
(plasticity.cuh:128-162) starts from its prediction instead of the
reference's max(eps_pl_dot dt sqrt(2/3), 1e-8) and still runs to the
reference tolerance.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

# record columns (sph_jc_log_enable)
SVM, EPS, EPSD, TEMP, NORM, DL, ITERS, DT = range(abi.JC_LOG_WIDTH)


class MlpError(RuntimeError):
    pass


def valid_records(records: np.ndarray) -> np.ndarray:
    """Logged return mappings with a usable target: |dev S_trial| > 0 and a
    positive increment.  A particle at the melting temperature has yield stress
    0 and may 'yield' with a zero deviator (the reference blanks it); its
    target is undefined."""
    r = np.asarray(records, np.float32)
    ok = (r[:, NORM] > 0) & (r[:, DL] > 0) & (r[:, SVM] > 0) & np.isfinite(r).all(1)
    return r[ok]


def features(records: np.ndarray, constants: abi.Constants):
    """Inputs x [n, 4] and target t [n] of logged return mappings.

    x = (log(svm / A), eps_pl, log(1 + eps_pl_dot / eps_dot_ref),
    (T - Tref) / (Tmelt - Tref)); t = log(2 G dl / |dev S_trial|), the log of
    the fraction of the trial deviator that the return removes."""
    r = np.asarray(records, np.float32)
    jc = constants.joco
    A = np.float32(jc.A)
    inv_ref = np.float32(1.0 / jc.eps_dot_ref)
    inv_dT = np.float32(1.0 / (jc.Tmelt - jc.Tref))
    x = np.empty((len(r), 4), np.float32)
    x[:, 0] = np.log(r[:, SVM] / A)
    x[:, 1] = r[:, EPS]
    x[:, 2] = np.log1p(r[:, EPSD] * inv_ref)
    x[:, 3] = (r[:, TEMP] - np.float32(jc.Tref)) * inv_dT
    two_mu = np.float32(2.0 * constants.phys.G)
    frac = np.maximum(two_mu * r[:, DL] / r[:, NORM], np.float32(1e-30))
    t = np.log(frac).astype(np.float32)
    return x, t


class Mlp:
    def __init__(self, device: int = 0, seed: int = 0):
        self.lib = abi.load()
        h = C.c_void_p()
        r = self.lib.sph_mlp_create(device, seed, C.byref(h))
        self.h = h
        if r != abi.SPH_OK:
            msg = self.lib.sph_mlp_last_error(h).decode() if h.value else ""
            self.close()
            raise MlpError(f"sph_mlp_create failed ({r}): {msg}")

    def _ck(self, r, what):
        if r != abi.SPH_OK:
            raise MlpError(f"{what} failed ({r}): {self.lib.sph_mlp_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.sph_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(abi.MLP_NPARAMS, np.float32)
        n = abi.MlpNorm()
        self._ck(self.lib.sph_mlp_get_params(self.h, abi.ptr(p), C.byref(n)), "sph_mlp_get_params")
        return p, n

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        self._ck(self.lib.sph_mlp_set_params(self.h, abi.ptr(p), C.byref(norm) if norm is not None else None),
                 "sph_mlp_set_params")

    def fit_norm(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        self._ck(self.lib.sph_mlp_fit_norm(self.h, abi.ptr(x), abi.ptr(t), len(t)), "sph_mlp_fit_norm")

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(len(x), np.float32)
        self._ck(self.lib.sph_mlp_predict(self.h, abi.ptr(x), len(x), abi.ptr(y)), "sph_mlp_predict")
        return y

    def predict_warp(self, x):
        """predict through the warp-per-sample form of the fused step's epilogue."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(len(x), np.float32)
        self._ck(self.lib.sph_mlp_predict_warp(self.h, abi.ptr(x), len(x), abi.ptr(y)), "sph_mlp_predict_warp")
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(abi.MLP_NPARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._ck(self.lib.sph_mlp_gradients(self.h, abi.ptr(x), abi.ptr(t), len(t), abi.ptr(g), abi.ptr(loss)),
                 "sph_mlp_gradients")
        return g, float(loss[0])

    def adam_step(self, x, t, lr):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = np.zeros(1, np.float32)
        self._ck(self.lib.sph_mlp_adam_step(self.h, abi.ptr(x), abi.ptr(t), len(t), lr, abi.ptr(loss)),
                 "sph_mlp_adam_step")
        return float(loss[0])

    def train(self, x, t, epochs=4, batch=8192, lr=1e-3, seed=0):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        losses = np.zeros(epochs, np.float32)
        self._ck(self.lib.sph_mlp_train(self.h, abi.ptr(x), abi.ptr(t), len(t), epochs, batch, lr, seed,
                                        abi.ptr(losses)), "sph_mlp_train")
        return losses
