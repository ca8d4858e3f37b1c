"""BatchSimulator: many independent physics-mode lattices advanced together (lbm_batch_*).

The reference runs one lattice per simulator; this is the batched form of the same step
for ensembles of lid-driven cavities and channels of uneven size.  Method "persistent"
runs all steps of a call in one cooperative launch replayed from a CUDA graph;
"tile_launches" launches once per step; "domain_loop" launches once per domain and step.
"""
import ctypes

import numpy as np

from . import _native as nat


def generate_domains(n: int, seed: int):
    """The seeded domain list (sides log-uniform 64..1024, aspect U[0.5,2], tau U[0.55,1],
    speed U[0.02,0.1], cavity or channel with probability 1/2)."""
    lib = nat.load()
    arr = (nat.DomainDesc * n)()
    nat.check(lib.lbm_batch_generate(int(n), int(seed), ctypes.cast(arr, ctypes.c_void_p)))
    scenes = {1: "cavity", 3: "channel"}
    return [dict(nx=d.nx, ny=d.ny, scene=scenes[d.scene], tau=d.tau, speed=d.speed) for d in arr]


class BatchSimulator:
    def __init__(self, domains):
        lib = nat.load()
        n = len(domains)
        arr = (nat.DomainDesc * n)()
        for a, d in zip(arr, domains):
            a.nx, a.ny = int(d["nx"]), int(d["ny"])
            a.scene = nat.SCENES[d["scene"]]
            a.tau, a.speed = float(d["tau"]), float(d["speed"])
        h = ctypes.c_void_p()
        nat.check(lib.lbm_batch_create(n, ctypes.cast(arr, ctypes.c_void_p), ctypes.byref(h)))
        self._lib, self._h = lib, h
        self.domains = [dict(d) for d in domains]
        nd, cells = ctypes.c_int32(), ctypes.c_uint64()
        nat.check(lib.lbm_batch_info(h, ctypes.byref(nd), ctypes.byref(cells)))
        self.cells = int(cells.value)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, cuda_stream: int):
        nat.check(self._lib.lbm_batch_set_stream(self._h, ctypes.c_void_p(cuda_stream or None)))

    @property
    def config(self) -> dict:
        c = nat.BatchConfig()
        nat.check(self._lib.lbm_batch_get_config(self._h, ctypes.byref(c)))
        inv = {v: k for k, v in nat.BATCH_METHODS.items()}
        return dict(tile_threads_x=c.tile_threads_x, tile_rows=c.tile_rows, blocks_per_sm=c.blocks_per_sm,
                    method=inv[c.method], ms_per_step=c.ms_per_step, cells_per_thread=c.cells_per_thread,
                    linear=bool(c.linear), full_occupancy=bool(c.full_occupancy))

    def configure(self, tile_threads_x=None, tile_rows=None, blocks_per_sm=None, method=None, cells_per_thread=None,
                  linear=None, full_occupancy=None):
        c = nat.BatchConfig()
        nat.check(self._lib.lbm_batch_get_config(self._h, ctypes.byref(c)))
        if tile_threads_x is not None:
            c.tile_threads_x = int(tile_threads_x)
        if tile_rows is not None:
            c.tile_rows = int(tile_rows)
        if blocks_per_sm is not None:
            c.blocks_per_sm = int(blocks_per_sm)
        if method is not None:
            c.method = nat.BATCH_METHODS[method]
        if cells_per_thread is not None:
            c.cells_per_thread = int(cells_per_thread)
        if linear is not None:
            c.linear = 1 if linear else 0
        if full_occupancy is not None:
            c.full_occupancy = 1 if full_occupancy else 0
        nat.check(self._lib.lbm_batch_set_config(self._h, ctypes.byref(c)))

    def tune(self, trial_steps: int = 20) -> dict:
        c = nat.BatchConfig()
        nat.check(self._lib.lbm_batch_tune(self._h, int(trial_steps), ctypes.byref(c)))
        return self.config

    def step(self, n: int = 1):
        nat.check(self._lib.lbm_batch_step(self._h, int(n)))

    def status(self):
        nat.check(self._lib.lbm_batch_status(self._h))

    def inject_missing_arrival(self, nsteps: int, block: int, step: int, timeout_ns: int = 0) -> int:
        """Returns the status code (LBM_ERR_TIMEOUT when the barrier timed out)."""
        return self._lib.lbm_batch_inject_missing_arrival(self._h, int(nsteps), int(block), int(step),
                                                          int(timeout_ns))

    def read_macro(self, i: int):
        d = self.domains[i]
        rho = np.empty((d["ny"], d["nx"]), np.float32)
        ux, uy = np.empty_like(rho), np.empty_like(rho)
        nat.check(self._lib.lbm_batch_read_macro(self._h, int(i), nat.ptr(rho), nat.ptr(ux), nat.ptr(uy)))
        return rho, ux, uy

    def read_populations(self, i: int) -> np.ndarray:
        d = self.domains[i]
        f = np.empty((9, d["ny"], d["nx"]), np.float32)
        nat.check(self._lib.lbm_batch_read_populations(self._h, int(i), nat.ptr(f)))
        return f

    def info(self, i: int) -> np.ndarray:
        d = self.domains[i]
        out = np.empty((d["ny"], d["nx"]), nat.INFO_DTYPE)
        nat.check(self._lib.lbm_batch_read_info(self._h, int(i), nat.ptr(out)))
        return out

    def conservation(self, i: int):
        out = (ctypes.c_double * 3)()
        nat.check(self._lib.lbm_batch_conservation(self._h, int(i), out))
        return tuple(float(v) for v in out)

    @property
    def counters(self):
        s, l = ctypes.c_uint64(), ctypes.c_uint64()
        nat.check(self._lib.lbm_batch_counters(self._h, ctypes.byref(s), ctypes.byref(l)))
        return int(s.value), int(l.value)
