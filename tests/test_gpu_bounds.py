"""The bounds-checked build (liblbm_bounds.so, LBM_BOUNDS_CHECK): every population, flag and
info index of the step kernels is compared with its buffer's extent; an out-of-range index is
recorded (lbm_bounds_report) and its access skipped, so nothing traps.  compute-sanitizer is
not available on these machines, so this build is the check that the index arithmetic stays
inside the buffers.

The child process loads the checked build (SIMUVERSE_LBM_VARIANT=bounds) and runs each kernel
family -- the reference-mode step (exact and fast), the one-cell physics step (FP32, FP64,
FP16), the tiled 16-bit step (global loads and rows staged in shared memory), the bulk-copy
step and the batched form -- over odd lattice sizes
(4x4, 5x7, 300x5, 1032x66 and the nearest sizes each kernel accepts) with obstacles on the
cells next to the walls and in the corners, inlet, outlet and forcing cells, for a few steps
with the macro field written every step; the record must stay empty.  The self-test first
shows that the record works: one index equal to its extent, evaluated without an access, is
counted.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

pytestmark = pytest.mark.gpu


def _wall_obstacles(info, seed):
    """Obstacles on cells next to the walls and in the corners, plus a few random ones."""
    ny, nx = info.shape
    rng = np.random.default_rng(seed)
    cand = [(1, 1), (nx - 2, 1), (1, ny - 2), (nx - 2, ny - 2), (nx // 2, 1), (nx // 2, ny - 2), (1, ny // 2)]
    cand += [(int(rng.integers(0, nx)), int(rng.integers(0, ny))) for _ in range(max(2, nx * ny // 200))]
    for x, y in cand:
        if 0 <= x < nx and 0 <= y < ny:
            info[y, x] = (4, -1, 0.0, 0.0)
    return info


def _forcing_cells(info, seed):
    ny, nx = info.shape
    rng = np.random.default_rng(seed + 1)
    for _ in range(3):
        x, y = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        if info[y, x]["material"] == 1:
            info[y, x] = (6, 5, 0.05, -0.02)
    return info


def _report(lib):
    import ctypes

    n, idx, lim, site = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_int32()
    rc = lib.lbm_bounds_report(ctypes.byref(n), ctypes.byref(idx), ctypes.byref(lim), ctypes.byref(site))
    assert rc == 0, lib.lbm_last_error()
    return n.value, idx.value, lim.value, site.value


def child_main():
    """Runs in the child process with the bounds-checked library."""
    from simuverse_gb300 import BatchSimulator, FluidSimulator, generate_domains
    from simuverse_gb300 import _native as nat

    lib = nat.load()
    assert nat.LIB_PATH.endswith("liblbm_bounds.so")
    assert lib.lbm_bounds_selftest() == 0, lib.lbm_last_error()
    n, idx, lim, site = _report(lib)
    assert (n, idx, lim, site) == (1, 7, 7, 99), (n, idx, lim, site)
    assert _report(lib)[0] == 0  # the report clears the record

    runs = 0

    def check(label):
        rec = _report(lib)
        assert rec[0] == 0, "%s: %d out-of-range indices, first %d of extent %d at site %d" % ((label,) + rec)

    # reference mode, both arithmetics
    for nx, ny in ((4, 4), (5, 7), (300, 5), (1032, 66), (131, 97)):
        for scene in ("custom", "cavity", "poiseuille"):
            for arith in ("exact", "fast"):
                s = FluidSimulator(nx, ny, mode="reference", scene=scene, tau=0.57, arith=arith, macro_every_step=True)
                info = _forcing_cells(_wall_obstacles(s.info(), nx * ny), nx)
                s.set_info(info)
                s.step(6)
                s.sync()
                s.close()
                check("reference %s %dx%d %s" % (arith, nx, ny, scene))
                runs += 1
    # physics mode, one-cell kernel (every collision for FP32)
    for nx, ny in ((4, 4), (5, 7), (300, 5), (1032, 66)):
        for scene in ("cavity", "channel", "periodic"):
            for dtype, coll in (("f32", "bgk"), ("f32", "kbc"), ("f32", "mrt"), ("f64", "bgk"), ("f16", "bgk")):
                s = FluidSimulator(nx, ny, mode="physics", scene=scene, dtype=dtype, collision=coll, kernel="cell",
                                   tau=0.6, lid_speed=0.05, inlet_speed=0.03, disk_radius=(1.0, 2.0),
                                   macro_every_step=True)
                info = _forcing_cells(_wall_obstacles(s.info(), nx + ny), ny)
                s.set_info(info)
                s.step(6)
                s.sync()
                s.close()
                check("physics cell %s %s %dx%d %s" % (dtype, coll, nx, ny, scene))
                runs += 1
    # tiled 16-bit kernel (nx % 64 == 0), both roundings
    for nx, ny in ((64, 4), (128, 5), (1024, 66)):
        for scene in ("cavity", "channel"):
            for dtype, rnd in (("f16", "nearest"), ("bf16", "stochastic")):
                s = FluidSimulator(nx, ny, mode="physics", scene=scene, dtype=dtype, kernel="tiled", rounding=rnd,
                                   tau=0.6, lid_speed=0.05, inlet_speed=0.03, disk_radius=(1.0, 2.0),
                                   macro_every_step=True)
                s.set_info(_forcing_cells(_wall_obstacles(s.info(), nx), ny))
                s.step(6)
                s.sync()
                s.close()
                check("tiled %s %dx%d %s" % (dtype, nx, ny, scene))
                runs += 1
    # the same layout stepped from rows staged in shared memory (strips of 8 tiles: 576 = 9 tiles)
    for nx, ny in ((64, 4), (576, 5), (1024, 66)):
        for scene in ("cavity", "channel"):
            for dtype, rnd in (("f16", "stochastic"), ("bf16", "nearest")):
                s = FluidSimulator(nx, ny, mode="physics", scene=scene, dtype=dtype, kernel="ring", rounding=rnd,
                                   tau=0.6, lid_speed=0.05, inlet_speed=0.03, disk_radius=(1.0, 2.0),
                                   macro_every_step=True)
                s.set_info(_forcing_cells(_wall_obstacles(s.info(), nx), ny))
                s.step(6)
                s.status()
                s.close()
                check("ring %s %dx%d %s" % (dtype, nx, ny, scene))
                runs += 1
    # bulk-copy kernel (nx % 8 == 0)
    for nx, ny in ((8, 4), (296, 7), (1032, 66), (520, 5)):
        for scene in ("cavity", "channel", "periodic"):
            for dtype in ("f32", "f64", "bf16"):
                s = FluidSimulator(nx, ny, mode="physics", scene=scene, dtype=dtype, kernel="bulk", tau=0.6,
                                   lid_speed=0.05, inlet_speed=0.03, disk_radius=(1.0, 2.0), macro_every_step=True)
                s.set_info(_forcing_cells(_wall_obstacles(s.info(), nx * 3), nx))
                s.step(6)
                s.status()
                s.close()
                check("bulk %s %dx%d %s" % (dtype, nx, ny, scene))
                runs += 1
    # batched form: every method on a seeded list with small domains
    doms = generate_domains(12, 77)
    b = BatchSimulator(doms)
    for method in ("persistent", "tile_launches", "domain_loop"):
        b.configure(method=method)
        b.step(4)
        b.status()
        check("batch %s" % method)
        runs += 1
    b.close()
    print("bounds-checked runs:", runs)


def test_bounds_checked_build_records_nothing(gpu):
    from simuverse_gb300 import build

    build.build(variant="bounds")
    env = dict(os.environ, SIMUVERSE_LBM_VARIANT="bounds")
    code = "import sys; sys.path[:0] = [%r, %r]; import test_gpu_bounds as t; t.child_main()" % (HERE, ROOT)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "bounds-checked runs:" in r.stdout


def test_normal_build_has_no_bounds_record(gpu):
    lib = gpu
    assert lib.lbm_bounds_report(None, None, None, None) == -6  # LBM_ERR_STATE
    assert lib.lbm_bounds_selftest() == -6
