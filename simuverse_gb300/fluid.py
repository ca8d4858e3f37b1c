"""FluidSimulator: the host-side mirror of simuverse's fluid simulator over liblbm.

Method names and semantics follow the reference's ``Simulator`` trait
(simuverse/src/lib.rs:72-106) as implemented by ``FluidSimulator``
(simuverse/src/fluid/fluid_simulator.rs:136-249):

=====================  ===========================================================
reference              here
=====================  ===========================================================
FluidSimulator::new    ``FluidSimulator(nx, ny, ...)``: the lattice is given
                       directly instead of being derived from a window
compute(encoder)       ``compute()``: one frame = two steps (swap 0 then 1)
reset(app)             ``reset()``
on_click(app, pos)     ``on_click(pos)``
touch_begin / _move    ``touch_begin()`` / ``touch_move(pos)``
update_uniforms        ``update_uniforms(viscosity)``
macro_tex              ``read_macro()`` / ``read_macro_rgba16f()``
=====================  ===========================================================

Requests the reference silently ignores (a click near the border, the first point of a
drag) return False; errors raise ``LbmError``.
"""
import ctypes

import numpy as np

from . import _native as nat


def make_params(nx: int, ny: int, *, mode: str = "reference", dtype: str = "f32", scene: str = "poiseuille",
                tau: float = None, viscosity: float = None, lid_speed: float = None, inlet_speed: float = None,
                solid_fraction: float = 0.05, disk_radius=(8.0, 32.0), seed: int = 0, pixel_size: int = 2,
                macro_every_step: bool = False, kernel: str = "auto", collision: str = "bgk",
                rounding: str = "nearest", arith: str = "exact") -> "nat.LbmParams":
    """lbm_params from keyword arguments (lbm_params_default for the rest)."""
    lib = nat.load()
    p = nat.LbmParams()
    lib.lbm_params_default(ctypes.byref(p))
    p.nx, p.ny = int(nx), int(ny)
    p.mode = nat.MODES[mode]
    p.dtype = nat.DTYPES[dtype]
    p.scene = nat.SCENES[scene]
    if tau is not None:
        p.tau = float(tau)
    elif viscosity is not None:
        p.tau = float(np.float32(3.0) * np.float32(viscosity) + np.float32(0.5))
    if lid_speed is not None:
        p.lid_speed = float(lid_speed)
    if inlet_speed is not None:
        p.inlet_speed = float(inlet_speed)
    p.solid_fraction = float(solid_fraction)
    p.disk_rmin, p.disk_rmax = float(disk_radius[0]), float(disk_radius[1])
    p.seed = int(seed)
    p.pixel_size = int(pixel_size)
    p.macro_every_step = 1 if macro_every_step else 0
    p.kernel = nat.KERNELS[kernel]
    p.collision = nat.COLLISIONS[collision]
    p.rounding = nat.ROUNDINGS[rounding]
    p.arith = nat.ARITHS[arith]
    return p


def scene_disks(nx: int, ny: int, **kw) -> np.ndarray:
    """The channel scene's disks as an (n, 3) array of (cx, cy, r) (lbm_scene_disks); empty for
    other scenes."""
    lib = nat.load()
    p = make_params(nx, ny, **kw)
    n = ctypes.c_int32()
    nat.check(lib.lbm_scene_disks(ctypes.byref(p), None, 0, ctypes.byref(n)))
    out = np.empty((n.value, 3), np.float64)
    if n.value:
        nat.check(lib.lbm_scene_disks(ctypes.byref(p), nat.ptr(out), n.value, ctypes.byref(n)))
    return out


def memory_set_retain(nbytes: int):
    """Bytes of device memory that destroyed lattices leave reserved in the library's pool of
    every device, for the next lattices (lbm_memory_set_retain)."""
    nat.check(nat.load().lbm_memory_set_retain(int(nbytes)))


def memory_trim():
    """Give the current device pool's unused memory back to the device (lbm_memory_trim)."""
    nat.check(nat.load().lbm_memory_trim())


def memory_stats() -> dict:
    """Reserved and used bytes of the current device's lattice pool (lbm_memory_stats)."""
    r, u = ctypes.c_uint64(), ctypes.c_uint64()
    nat.check(nat.load().lbm_memory_stats(ctypes.byref(r), ctypes.byref(u)))
    return {"reserved": r.value, "used": u.value}


class FluidSimulator:
    def __init__(self, nx: int, ny: int, **kw):
        """An nx x ny lattice (lbm_create).  Keywords, all optional (make_params): mode
        ("reference" | "physics"), dtype ("f32" | "f64" | "f16" | "bf16"), scene ("poiseuille" |
        "cavity" | "custom" | "channel" | "periodic"), tau or viscosity, lid_speed, inlet_speed,
        solid_fraction, disk_radius, seed, pixel_size, macro_every_step, kernel, collision,
        rounding ("nearest" | "stochastic"), arith ("exact" | "fast": reference-mode rounding)."""
        lib = nat.load()
        p = make_params(nx, ny, **kw)
        mode, dtype, scene = kw.get("mode", "reference"), kw.get("dtype", "f32"), kw.get("scene", "poiseuille")
        rounding, pixel_size = kw.get("rounding", "nearest"), kw.get("pixel_size", 2)
        h = ctypes.c_void_p()
        nat.check(lib.lbm_create(ctypes.byref(p), ctypes.byref(h)))
        self._lib = lib
        self._h = h
        self.nx, self.ny = int(nx), int(ny)
        self.N = self.nx * self.ny
        self.mode, self.dtype, self.scene = mode, dtype, scene
        self.rounding = rounding
        self.pixel_size = int(pixel_size)

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def set_stream(self, cuda_stream: int):
        """Queue the simulator's work on a caller-owned CUDA stream (0 restores its own)."""
        nat.check(self._lib.lbm_set_stream(self._h, ctypes.c_void_p(cuda_stream or None)))

    # ------------------------------------------------------------------ stepping
    def step(self, n: int = 1):
        nat.check(self._lib.lbm_step(self._h, int(n)))

    def compute(self):
        nat.check(self._lib.lbm_compute(self._h))

    def reset(self):
        nat.check(self._lib.lbm_reset(self._h))

    def update_uniforms(self, viscosity: float):
        nat.check(self._lib.lbm_update_viscosity(self._h, float(viscosity)))

    def set_tau(self, tau: float):
        nat.check(self._lib.lbm_set_tau(self._h, float(tau)))

    @property
    def tau(self) -> float:
        p = nat.LbmParams()
        nat.check(self._lib.lbm_get_params(self._h, ctypes.byref(p)))
        return p.tau

    # ------------------------------------------------------------------ interaction
    def on_click(self, pos) -> bool:
        return nat.check(self._lib.lbm_on_click(self._h, float(pos[0]), float(pos[1]))) == nat.LBM_OK

    def add_obstacle(self, x: int, y: int):
        nat.check(self._lib.lbm_add_obstacle(self._h, int(x), int(y)))

    def touch_begin(self):
        nat.check(self._lib.lbm_touch_begin(self._h))

    def touch_move(self, pos) -> bool:
        return nat.check(self._lib.lbm_touch_move(self._h, float(pos[0]), float(pos[1]))) == nat.LBM_OK

    def add_external_force(self, pos, pre_pos):
        nat.check(self._lib.lbm_add_external_force(self._h, float(pos[0]), float(pos[1]),
                                                   float(pre_pos[0]), float(pre_pos[1])))

    # ------------------------------------------------------------------ mask
    def info(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), dtype=nat.INFO_DTYPE)
        nat.check(self._lib.lbm_get_info(self._h, nat.ptr(out)))
        return out

    def set_info(self, info: np.ndarray):
        info = np.ascontiguousarray(info, dtype=nat.INFO_DTYPE).reshape(self.ny, self.nx)
        nat.check(self._lib.lbm_set_info(self._h, nat.ptr(info)))

    def apply_edits(self, edits) -> int:
        """Batched interaction on the GPU (lbm_apply_edits): edits is a list of tuples
        (kind, *args) with kind in obstacle (x, y), click (px, py), force (pos_x, pos_y, pre_x,
        pre_y), touch_begin (), touch_move (px, py).  Returns the number of mask writes."""
        arr = (nat.Edit * max(1, len(edits)))()
        for i, e in enumerate(edits):
            arr[i].kind = nat.EDITS[e[0]]
            vals = list(e[1:]) + [0.0] * (4 - len(e[1:]))
            arr[i].a, arr[i].b, arr[i].c, arr[i].d = (float(v) for v in vals)
        n = ctypes.c_int32()
        nat.check(self._lib.lbm_apply_edits(self._h, arr, len(edits), ctypes.byref(n)))
        return n.value

    # ------------------------------------------------------------------ fields
    def read_macro(self, out=None):
        """(rho, ux, uy) of the last step as (ny, nx) float32 arrays; `out` = three C-contiguous
        float32 arrays of nx * ny values to fill (page-locked ones copy fastest)."""
        if out is None:
            out = tuple(np.empty((self.ny, self.nx), np.float32) for _ in range(3))
        for a in out:
            if a.dtype != np.float32 or a.size != self.N or not a.flags.c_contiguous:
                raise ValueError("read_macro needs C-contiguous float32 arrays of nx*ny values")
        rho, ux, uy = out
        nat.check(self._lib.lbm_read_macro(self._h, nat.ptr(rho), nat.ptr(ux), nat.ptr(uy)))
        return rho, ux, uy

    def read_macro_rgba16f(self) -> np.ndarray:
        """macro_tex texels (ux, uy, rho, w) as float16, shape (ny, nx, 4)."""
        out = np.empty((self.ny, self.nx, 4), np.uint16)
        nat.check(self._lib.lbm_read_macro_rgba16f(self._h, nat.ptr(out)))
        return out.view(np.float16)

    def read_populations(self, dtype=np.float32) -> np.ndarray:
        """Absolute populations f_i, shape (9, ny, nx)."""
        dt = np.dtype(dtype)
        code = nat.DTYPES["f64"] if dt == np.float64 else nat.DTYPES["f32"]
        out = np.empty((9, self.ny, self.nx), dt if dt == np.float64 else np.float32)
        nat.check(self._lib.lbm_read_populations(self._h, nat.ptr(out), code))
        return out

    def write_populations(self, f: np.ndarray):
        f = np.ascontiguousarray(f)
        if f.dtype == np.float64:
            code = nat.DTYPES["f64"]
        else:
            f = f.astype(np.float32, copy=False)
            code = nat.DTYPES["f32"]
        if f.size != 9 * self.N:
            raise ValueError("expected 9*nx*ny populations")
        nat.check(self._lib.lbm_write_populations(self._h, nat.ptr(f), code))

    def init_equilibrium(self, rho=None, ux=None, uy=None):
        arrs = []
        for a in (rho, ux, uy):
            arrs.append(None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(self.ny, self.nx))
        ptrs = [None if a is None else nat.ptr(a) for a in arrs]
        nat.check(self._lib.lbm_init_equilibrium(self._h, *ptrs))

    # ------------------------------------------------------------------ diagnostics
    def conservation(self):
        out = (ctypes.c_double * 3)()
        nat.check(self._lib.lbm_conservation(self._h, out))
        return float(out[0]), float(out[1]), float(out[2])

    def nonfinite_count(self) -> int:
        n = ctypes.c_uint64(0)
        rc = self._lib.lbm_check_finite(self._h, ctypes.byref(n))
        if rc not in (nat.LBM_OK, nat.LBM_ERR_NAN):
            nat.check(rc)
        return int(n.value)

    def sync(self):
        """Wait for the handle's stream (lbm_status)."""
        self.status()

    def status(self):
        """Raises LbmError(LBM_ERR_TIMEOUT) if a step kernel gave up on a bounded wait."""
        nat.check(self._lib.lbm_status(self._h))

    def check_finite(self):
        n = ctypes.c_uint64(0)
        nat.check(self._lib.lbm_check_finite(self._h, ctypes.byref(n)))

    def macro_error(self, ref: "FluidSimulator"):
        """(rel L2 rho, rel L2 u, max |du|, max |drho|) of this field against ref's."""
        out = (ctypes.c_double * 4)()
        nat.check(self._lib.lbm_macro_error(self._h, ref._h, out))
        return tuple(float(v) for v in out)

    def save(self, path: str):
        nat.check(self._lib.lbm_save(self._h, path.encode()))

    def load(self, path: str):
        nat.check(self._lib.lbm_load(self._h, path.encode()))

    @property
    def steps_done(self) -> int:
        n = ctypes.c_uint64(0)
        nat.check(self._lib.lbm_steps_done(self._h, ctypes.byref(n)))
        return int(n.value)

    @property
    def kernel_launches(self) -> int:
        n = ctypes.c_uint64(0)
        nat.check(self._lib.lbm_kernel_launches(self._h, ctypes.byref(n)))
        return int(n.value)

    def device_populations(self):
        """(device pointer, tiled) of the population buffer the next step reads, in the
        handle's storage format; valid until the next step, reset, load or close."""
        p, t = ctypes.c_void_p(), ctypes.c_int32()
        nat.check(self._lib.lbm_device_populations(self._h, ctypes.byref(p), ctypes.byref(t)))
        return p.value, bool(t.value)

    def device_macro(self):
        """Device pointers (rho, ux, uy) of the macro planes, for in-GPU consumers."""
        r, u, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        nat.check(self._lib.lbm_device_macro(self._h, ctypes.byref(r), ctypes.byref(u), ctypes.byref(v)))
        return r.value, u.value, v.value
