"""Closure: the learned correction of a 4x-coarsened lattice (lbm_closure_*).

A three-layer 3x3 convolution (9 -> 32 -> 32 -> 9 channels, BF16 weights and activations,
FP32 accumulation on the tensor cores) maps the non-equilibrium part of a coarse cell's
populations to a correction of those populations, projected so that no cell's density or
momentum changes.  It is trained on the GPU (the library's own forward, backward and Adam
kernels) on pairs (coarse state after k coarse steps, coarse-grained fine state k*factor
fine steps later).
"""
import ctypes

import numpy as np

from . import _native as nat


def coarsen(fine, coarse, factor: int, neq_scale: float):
    """Write the coarse-grained state of FluidSimulator `fine` into `coarse`."""
    nat.check(nat.load().lbm_coarsen(fine.handle, coarse.handle, int(factor), float(neq_scale)))


class Closure:
    def __init__(self, nx: int, ny: int, seed: int = 0, s_in: float = 1000.0, s_out: float = 1000.0):
        lib = nat.load()
        h = ctypes.c_void_p()
        nat.check(lib.lbm_closure_create(int(nx), int(ny), int(seed), ctypes.byref(h)))
        self._lib, self._h = lib, h
        self.nx, self.ny = int(nx), int(ny)
        self.nparams = lib.lbm_closure_param_count()
        self.set_scales(s_in, s_out)
        self.crop = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_closure_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scales(self, s_in: float, s_out: float):
        nat.check(self._lib.lbm_closure_set_scales(self._h, float(s_in), float(s_out)))
        self.s_in, self.s_out = float(s_in), float(s_out)

    @property
    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, np.float32)
        nat.check(self._lib.lbm_closure_get_params(self._h, nat.ptr(out)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        nat.check(self._lib.lbm_closure_set_params(self._h, nat.ptr(p)))

    def apply(self, sim):
        """Correct the current populations of FluidSimulator `sim` in place."""
        nat.check(self._lib.lbm_closure_apply(self._h, sim.handle))

    def predict(self, sim) -> np.ndarray:
        """The correction the closure would add to `sim`, shape (9, ny, nx)."""
        out = np.empty((9, self.ny, self.nx), np.float32)
        nat.check(self._lib.lbm_closure_predict(self._h, sim.handle, nat.ptr(out)))
        return out

    def reserve(self, max_pairs: int, crop: int, batch: int):
        nat.check(self._lib.lbm_closure_reserve(self._h, int(max_pairs), int(crop), int(batch)))
        self.crop = int(crop)

    def add_pair(self, pred, target, ox: int, oy: int):
        nat.check(self._lib.lbm_closure_add_pair(self._h, pred.handle, target.handle, int(ox), int(oy)))

    @property
    def npairs(self) -> int:
        n = ctypes.c_int32()
        nat.check(self._lib.lbm_closure_pairs(self._h, ctypes.byref(n)))
        return int(n.value)

    def train(self, iters: int, lr: float = 1e-3, seed: int = 0) -> float:
        loss = ctypes.c_double()
        nat.check(self._lib.lbm_closure_train(self._h, int(iters), float(lr), int(seed), ctypes.byref(loss)))
        return float(loss.value)

    def eval(self, begin: int, end: int) -> float:
        loss = ctypes.c_double()
        nat.check(self._lib.lbm_closure_eval(self._h, int(begin), int(end), ctypes.byref(loss)))
        return float(loss.value)

    def loss_grad(self, feats: np.ndarray, targets: np.ndarray):
        """Mean loss and logical gradient for host crops feats/targets of shape (n, S, S, 9)."""
        feats = np.ascontiguousarray(feats, np.float32)
        targets = np.ascontiguousarray(targets, np.float32)
        n, S = feats.shape[0], feats.shape[1]
        loss = ctypes.c_double()
        g = np.empty(self.nparams, np.float32)
        nat.check(self._lib.lbm_closure_loss_grad(self._h, n, S, nat.ptr(feats), nat.ptr(targets), ctypes.byref(loss),
                                                  nat.ptr(g)))
        return float(loss.value), g
