"""TEST INFRASTRUCTURE, NOT PRODUCT CODE.

ctypes wrapper over oracle/lbm_oracle.c, the CPU restatement of simuverse's D2Q9 path.
Only tests/, ``__graft_entry__.smoke()`` (to check results) and bench.py's CPU-baseline leg
use it.  Parity status: UNPINNED -- the reference (Rust + WGSL on wgpu) cannot run on
these machines and its own tests hold no vectors for this path; see lbm_oracle.h.
"""
import ctypes
import os

import numpy as np

from . import build as _build

INFO_DTYPE = np.dtype([("material", "<i4"), ("block_iter", "<i4"), ("vx", "<f4"), ("vy", "<f4")])
SCENES = {"poiseuille": 0, "cavity": 1, "custom": 2}

_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        sig = {
            "lo_mask_reference": ([_I, _I, _I, _F, _F, _P], None),
            "lo_ref_init": ([_I, _I, _I, _P, _P, _P], None),
            "lo_ref_step": ([_I, _I, _F, _P, _P, _P, _P, _P], None),
            "lo_add_obstacle": ([_I, _I, _P, _P, _I, _I], _I),
            "lo_on_click": ([_I, _I, _I, _P, _P, _F, _F], _I),
            "lo_add_external_force": ([_I, _I, _I, _P, _F, _F, _F, _F], None),
            "lo_phys_step_f32": ([_I, _I, _F, _P, _P, _P, _P, _I], None),
            "lo_phys_step_f64": ([_I, _I, _D, _P, _P, _P, _P, _I], None),
            "lo_phys_init_f32": ([_I, _I, _P, _P, _P, _P, _P], None),
            "lo_phys_init_f64": ([_I, _I, _P, _P, _P, _P, _P], None),
            "lo_mask_physics_cavity": ([_I, _I, _F, _P], None),
            "lo_mask_physics_channel": ([_I, _I, _F, ctypes.c_uint64, _F, _F, _F, _P], _I),
            "lo_conservation_dev_f32": ([_I, _I, _P, _P, _P], None),
            "lo_conservation_dev_f64": ([_I, _I, _P, _P, _P], None),
            "lo_h16": ([_F], _F),
            "lo_particles_grid": ([_I, _I, _I, _P, _P], None),
            "lo_particles_init": ([_I, _I, _I, _I, _F, ctypes.c_uint64, _P], None),
            "lo_particles_update": ([_I, _I, _P, _P, _I, _F, _F, _F, _I, _I, _I, _I, _I, _P, _P], None),
            "lo_present_canvas": ([_I, _I, _I, _F, _P, _P, _P], None),
            "lo_curl": ([_I, _I, _P, _P, _I, _P], None),
            "lo_colorize": ([_I, _I, _P, _P, _P, _P, _I, _I, _I, _P], None),
            "lo_num_threads": ([], _I),
            "lo_set_num_threads": ([_I], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def mask_reference(nx, ny, scene, lid_vx=0.13, inlet_vx=0.12):
    info = np.zeros((ny, nx), INFO_DTYPE)
    lib().lo_mask_reference(nx, ny, SCENES[scene] if isinstance(scene, str) else scene, lid_vx, inlet_vx, _p(info))
    return info


def mask_physics_cavity(nx, ny, lid_vx):
    info = np.zeros((ny, nx), INFO_DTYPE)
    lib().lo_mask_physics_cavity(nx, ny, lid_vx, _p(info))
    return info


def mask_physics_channel(nx, ny, u_max, seed, solid_fraction=0.05, rmin=8.0, rmax=32.0):
    info = np.zeros((ny, nx), INFO_DTYPE)
    n = lib().lo_mask_physics_channel(nx, ny, u_max, seed, solid_fraction, rmin, rmax, _p(info))
    return info, n


def mask_periodic(nx, ny):
    info = np.zeros((ny, nx), INFO_DTYPE)
    info["material"] = 1
    info["block_iter"] = -1
    return info


class RefOracle:
    """Reference-mode oracle holding the same state the WGSL path holds."""

    def __init__(self, nx, ny, scene="poiseuille", tau=0.56, lid_vx=0.13, inlet_vx=0.12, pixel_size=2, info=None):
        self.nx, self.ny = nx, ny
        self.scene = scene
        self.lid_vx, self.inlet_vx = lid_vx, inlet_vx
        self.pixel_size = pixel_size
        self.fluid_ty = 1 if scene == "cavity" else 0
        self.set_tau(tau)
        self.info = mask_reference(nx, ny, scene, lid_vx, inlet_vx) if info is None else info.copy()
        self.host_info = self.info.copy()
        self.bufs = [np.zeros((9, ny, nx), np.float32), np.zeros((9, ny, nx), np.float32)]
        self.scratch = np.zeros(9 * nx * ny, np.float32)
        self.macro4 = np.zeros((ny, nx, 4), np.float32)
        self.pre = (0.0, 0.0)
        self._init()

    def set_tau(self, tau):
        self.tau = np.float32(tau)
        self.omega = np.float32(1.0) / self.tau

    def update_uniforms(self, viscosity):
        self.set_tau(np.float32(3.0) * np.float32(viscosity) + np.float32(0.5))

    def _init(self):
        lib().lo_ref_init(self.nx, self.ny, self.fluid_ty, _p(self.info), _p(self.bufs[0]), _p(self.bufs[1]))
        self.cur = 0
        self.macro4[...] = 0.0
        self.macro4[..., 3] = 1.0

    def reset(self):
        if self.scene == "poiseuille":
            self.info = mask_reference(self.nx, self.ny, self.scene, self.lid_vx, self.inlet_vx)
            self.host_info = self.info.copy()
        self._init()
        self.pre = (0.0, 0.0)

    def step(self, n=1):
        L = lib()
        for _ in range(n):
            L.lo_ref_step(self.nx, self.ny, float(self.omega), _p(self.info), _p(self.bufs[self.cur]),
                          _p(self.bufs[self.cur ^ 1]), _p(self.macro4), _p(self.scratch))
            self.cur ^= 1

    def compute(self):
        self.step(2)

    @property
    def populations(self):
        return self.bufs[self.cur]

    def macro(self):
        return self.macro4[..., 2].copy(), self.macro4[..., 0].copy(), self.macro4[..., 1].copy()

    def add_obstacle(self, x, y):
        return lib().lo_add_obstacle(self.nx, self.ny, _p(self.host_info), _p(self.info), x, y)

    def on_click(self, px, py):
        return lib().lo_on_click(self.nx, self.ny, self.pixel_size, _p(self.host_info), _p(self.info), px, py)

    def add_external_force(self, pos, pre):
        lib().lo_add_external_force(self.nx, self.ny, self.pixel_size, _p(self.info), pos[0], pos[1], pre[0], pre[1])

    def touch_begin(self):
        self.pre = (0.0, 0.0)

    def touch_move(self, pos):
        """fluid_simulator.rs:158-173 in float32 arithmetic."""
        px, py = np.float32(pos[0]), np.float32(pos[1])
        if px <= 0 or py <= 0:
            self.pre = (0.0, 0.0)
            return False
        dx = px - np.float32(self.pre[0])
        dy = py - np.float32(self.pre[1])
        dis = np.sqrt(dx * dx + dy * dy, dtype=np.float32)
        if (self.pre[0] == 0.0 and self.pre[1] == 0.0) or dis > np.float32(300.0):
            self.pre = (float(px), float(py))
            return False
        self.add_external_force((float(px), float(py)), self.pre)
        self.pre = (float(px), float(py))
        return True


class PhysOracle:
    """Physics-mode oracle (f32 or f64), deviation storage d = f - w."""

    W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)

    def __init__(self, info, tau, dtype=np.float32, collision=0):
        self.collision = int(collision)
        self.info = np.ascontiguousarray(info, INFO_DTYPE).copy()
        self.ny, self.nx = self.info.shape
        self.dtype = np.dtype(dtype)
        self.set_tau(tau)
        self.bufs = [np.zeros((9, self.ny, self.nx), self.dtype), np.zeros((9, self.ny, self.nx), self.dtype)]
        self.macro3 = np.zeros((3, self.ny, self.nx), self.dtype)
        self.init_equilibrium()

    def set_tau(self, tau):
        # the library takes tau as FP32; FP64 runs use 1 / double(tau)
        if self.dtype == np.float32:
            self.omega = float(np.float32(1.0) / np.float32(tau))
        else:
            self.omega = 1.0 / float(np.float32(tau))

    def _sfx(self):
        return "f32" if self.dtype == np.float32 else "f64"

    def init_equilibrium(self, rho=None, ux=None, uy=None):
        conv = [None if a is None else np.ascontiguousarray(a, self.dtype) for a in (rho, ux, uy)]
        getattr(lib(), "lo_phys_init_" + self._sfx())(self.nx, self.ny, _p(self.info), *[_p(a) for a in conv],
                                                       _p(self.bufs[0]))
        self.bufs[1][...] = self.bufs[0]
        self.cur = 0

    def step(self, n=1):
        fn = getattr(lib(), "lo_phys_step_" + self._sfx())
        for _ in range(n):
            fn(self.nx, self.ny, self.omega, _p(self.info), _p(self.bufs[self.cur]), _p(self.bufs[self.cur ^ 1]),
               _p(self.macro3), self.collision)
            self.cur ^= 1

    @property
    def deviations(self):
        return self.bufs[self.cur]

    def populations(self, dtype=np.float64):
        w = self.W.astype(dtype).reshape(9, 1, 1)
        return self.bufs[self.cur].astype(dtype) + w

    def macro(self):
        return self.macro3[0].copy(), self.macro3[1].copy(), self.macro3[2].copy()

    def conservation(self):
        out = (ctypes.c_double * 3)()
        getattr(lib(), "lo_conservation_dev_" + self._sfx())(self.nx, self.ny, _p(self.info), _p(self.bufs[self.cur]),
                                                              out)
        return float(out[0]), float(out[1]), float(out[2])


def num_threads():
    return lib().lo_num_threads()


def set_num_threads(n):
    lib().lo_set_num_threads(int(n))


# ---------------------------------------------------------------------------------------
# consumers of the macro field (lbm_oracle_view.inc)
# ---------------------------------------------------------------------------------------
def particles_grid(cw, ch, count):
    a, b = ctypes.c_int(), ctypes.c_int()
    lib().lo_particles_grid(cw, ch, count, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def particles_init(cw, ch, num_x, num_y, life_time, seed):
    out = np.empty((num_x * num_y, 6), np.float32)
    lib().lo_particles_init(cw, ch, num_x, num_y, float(life_time), int(seed), _p(out))
    return out


def particles_update(ux, uy, zero, lattice_pixel, life_time, speed_factor, point_size, cw, ch, poiseuille, state,
                     canvas):
    """One particle_update.wgsl pass; state (n, 6) and canvas (ch, cw, 3) float32, in place."""
    ny, nx = ux.shape
    ux = np.ascontiguousarray(ux, np.float32)
    uy = np.ascontiguousarray(uy, np.float32)
    assert state.dtype == np.float32 and state.flags.c_contiguous and canvas.dtype == np.float32
    lib().lo_particles_update(nx, ny, _p(ux), _p(uy), int(zero), float(lattice_pixel), float(life_time),
                              float(speed_factor), int(point_size), cw, ch, int(poiseuille), state.shape[0],
                              _p(state), _p(canvas))


def present_canvas(canvas, color_ty, speed_ty, fade_out, rgb=(1.0, 1.0, 1.0)):
    """present.wgsl over the canvas (ch, cw, 3) in place; returns RGBA (ch, cw, 4)."""
    ch, cw, _ = canvas.shape
    rgba = np.empty((ch, cw, 4), np.float32)
    col = np.asarray(rgb, np.float32)
    lib().lo_present_canvas(cw * ch, int(color_ty), int(speed_ty), float(fade_out), _p(col), _p(canvas), _p(rgba))
    return rgba


def curl(ux, uy, zero=False):
    ny, nx = ux.shape
    ux = np.ascontiguousarray(ux, np.float32)
    uy = np.ascontiguousarray(uy, np.float32)
    out = np.empty((ny, nx), np.float32)
    lib().lo_curl(nx, ny, _p(ux), _p(uy), int(zero), _p(out))
    return out


def colorize(rho, ux, uy, curl_field, cw, ch, mode, zero=False):
    """mode 0: curl hue, 1: velocity-angle hue; fields are the FP32 macro planes."""
    ny, nx = ux.shape
    planes = []
    for a in (rho, ux, uy):
        a = np.zeros((ny, nx), np.float32) if zero else np.asarray(a, np.float32).astype(np.float16).astype(np.float32)
        planes.append(np.ascontiguousarray(a))
    c = None if curl_field is None else np.ascontiguousarray(curl_field, np.float32)
    rgba = np.empty((ch, cw, 4), np.float32)
    lib().lo_colorize(nx, ny, _p(planes[0]), _p(planes[1]), _p(planes[2]), _p(c), cw, ch, int(mode), _p(rgba))
    return rgba
