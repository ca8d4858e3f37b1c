"""Consumers of the macro field on the device: tracer particles with their splat canvas,
the canvas presentation, the curl field and the field colour maps (lbm_particles_*,
lbm_curl, lbm_colorize of include/lbm.h).

simuverse runs these after each lattice step (FluidSimulator::compute in
simuverse/src/fluid/fluid_simulator.rs:217-232: step, particle update, step, particle
update) and draws the canvas with present.wgsl.  Here everything stays in device memory;
read-back functions copy to numpy for inspection and tests.
"""
import ctypes

import numpy as np

from . import _native as nat


def particle_params(canvas_w, canvas_h, **kw) -> "nat.ParticleParams":
    p = nat.ParticleParams()
    nat.load().lbm_particle_params_default(ctypes.byref(p))
    p.canvas_w, p.canvas_h = int(canvas_w), int(canvas_h)
    for k, v in kw.items():
        if k == "color":
            for i, c in enumerate(v):
                p.color[i] = float(c)
        else:
            setattr(p, k, v)
    return p


def particles_grid(canvas_w, canvas_h, count):
    a, b = ctypes.c_int32(), ctypes.c_int32()
    nat.check(nat.load().lbm_particles_grid(int(canvas_w), int(canvas_h), int(count), ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


class Particles:
    """Tracer particles advected by the macro field of a FluidSimulator."""

    def __init__(self, sim, canvas_w=None, canvas_h=None, **kw):
        lib = nat.load()
        cw = sim.nx * sim.pixel_size if canvas_w is None else canvas_w
        ch = sim.ny * sim.pixel_size if canvas_h is None else canvas_h
        self.params = particle_params(cw, ch, **kw)
        h = ctypes.c_void_p()
        nat.check(lib.lbm_particles_create(sim.handle, ctypes.byref(self.params), ctypes.byref(h)))
        self._lib, self._h, self.sim = lib, h, sim
        self.canvas_w, self.canvas_h = int(cw), int(ch)
        a, b = ctypes.c_int32(), ctypes.c_int32()
        nat.check(lib.lbm_particles_info(h, ctypes.byref(a), ctypes.byref(b)))
        self.num_x, self.num_y = a.value, b.value
        self.count = self.num_x * self.num_y

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_particles_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self):
        nat.check(self._lib.lbm_particles_update(self._h, self.sim.handle))

    def present(self) -> int:
        """Colour the canvas and fade it; returns the device pointer of the RGBA buffer."""
        p = ctypes.c_void_p()
        nat.check(self._lib.lbm_particles_present(self._h, self.sim.handle, ctypes.byref(p)))
        return p.value

    def compute(self):
        """The reference's per-frame compute: step, update, step, update."""
        for _ in range(2):
            self.sim.step(1)
            self.update()

    def state(self) -> np.ndarray:
        out = np.empty((self.count, 6), np.float32)
        nat.check(self._lib.lbm_particles_read(self._h, nat.ptr(out)))
        return out

    def set_state(self, s: np.ndarray):
        s = np.ascontiguousarray(s, np.float32)
        assert s.shape == (self.count, 6)
        nat.check(self._lib.lbm_particles_write(self._h, nat.ptr(s)))

    def canvas(self) -> np.ndarray:
        out = np.empty((self.canvas_h, self.canvas_w, 3), np.float32)
        nat.check(self._lib.lbm_particles_read_canvas(self._h, nat.ptr(out), None))
        return out

    def rgba(self) -> np.ndarray:
        out = np.empty((self.canvas_h, self.canvas_w, 4), np.float32)
        nat.check(self._lib.lbm_particles_read_canvas(self._h, None, nat.ptr(out)))
        return out

    def counters(self):
        u, l = ctypes.c_uint64(), ctypes.c_uint64()
        nat.check(self._lib.lbm_particles_counters(self._h, ctypes.byref(u), ctypes.byref(l)))
        return u.value, l.value


def curl(sim, out_device=None) -> np.ndarray:
    """curl_update.wgsl of the current macro field; (ny, nx) float32 (FP16-rounded values).
    With out_device (a torch tensor of nx*ny float32 on the lattice's GPU) the result
    stays there and None is returned."""
    import torch

    t = out_device if out_device is not None else torch.empty(sim.ny * sim.nx, dtype=torch.float32, device="cuda")
    nat.check(nat.load().lbm_curl(sim.handle, ctypes.c_void_p(t.data_ptr())))
    if out_device is not None:
        return None
    sim.sync()
    return t.cpu().numpy().reshape(sim.ny, sim.nx)


def colorize(sim, mode="curl", canvas_w=None, canvas_h=None) -> np.ndarray:
    """Field colour map (LBM_COLOR_CURL or LBM_COLOR_ANGLE) as (canvas_h, canvas_w, 4) RGBA."""
    import torch

    cw = sim.nx * sim.pixel_size if canvas_w is None else int(canvas_w)
    ch = sim.ny * sim.pixel_size if canvas_h is None else int(canvas_h)
    lib = nat.load()
    c = None
    if nat.COLOR_MODES[mode] == 0:
        c = torch.empty(sim.ny * sim.nx, dtype=torch.float32, device="cuda")
        nat.check(lib.lbm_curl(sim.handle, ctypes.c_void_p(c.data_ptr())))
    out = torch.empty(ch * cw * 4, dtype=torch.float32, device="cuda")
    nat.check(lib.lbm_colorize(sim.handle, nat.COLOR_MODES[mode], None if c is None else ctypes.c_void_p(c.data_ptr()),
                               cw, ch, ctypes.c_void_p(out.data_ptr())))
    sim.sync()
    return out.cpu().numpy().reshape(ch, cw, 4)
