"""Physics-mode scene masks built on the device equal the host builder's records bit for bit
(lbm_build_mask, itself checked against the oracle), and the host copy that the reference's
edit paths use, built from the parameters on first use, stays consistent: obstacles added
after creation, checkpoints and resets give the same records as a host-built mask."""
import ctypes

import numpy as np
import pytest

from simuverse_gb300 import FluidSimulator
from simuverse_gb300 import _native as nat

pytestmark = pytest.mark.gpu

CASES = [
    ("channel", 256, 96, 5, 0.05, (4.0, 9.0)),
    ("channel", 333, 127, 77, 0.08, (3.0, 12.0)),
    ("channel", 1024, 512, 1234, 0.05, (8.0, 32.0)),
    ("cavity", 100, 70, 0, 0.05, (8.0, 32.0)),
    ("periodic", 64, 48, 0, 0.05, (8.0, 32.0)),
]


def _kw(scene, seed, frac, radius):
    return dict(mode="physics", scene=scene, tau=0.6, lid_speed=0.1, inlet_speed=0.05, seed=seed,
                solid_fraction=frac, disk_radius=radius)


def _host_mask(nx, ny, **kw):
    lib = nat.load()
    p = nat.LbmParams()
    lib.lbm_params_default(ctypes.byref(p))
    p.nx, p.ny, p.mode, p.scene = nx, ny, 1, nat.SCENES[kw["scene"]]
    p.tau, p.lid_speed, p.inlet_speed = kw["tau"], kw["lid_speed"], kw["inlet_speed"]
    p.seed, p.solid_fraction = kw["seed"], kw["solid_fraction"]
    p.disk_rmin, p.disk_rmax = kw["disk_radius"]
    out = np.empty((ny, nx), dtype=nat.INFO_DTYPE)
    nat.check(lib.lbm_build_mask(ctypes.byref(p), nat.ptr(out)))
    return out


@pytest.mark.parametrize("scene,nx,ny,seed,frac,radius", CASES)
def test_device_scene_equals_host_mask(gpu, scene, nx, ny, seed, frac, radius):
    kw = _kw(scene, seed, frac, radius)
    sim = FluidSimulator(nx, ny, **kw)
    host = _host_mask(nx, ny, **kw)
    dev = sim.info()
    assert np.array_equal(dev.view(np.uint8), host.view(np.uint8))
    if scene == "channel":
        assert np.count_nonzero(dev["material"] == 4) >= frac * nx * ny
    sim.close()


def test_obstacle_after_device_scene_matches_host_edit(gpu):
    nx, ny = 256, 128
    kw = _kw("channel", 9, 0.05, (4.0, 9.0))
    sim = FluidSimulator(nx, ny, **kw)
    sim.add_obstacle(120, 64)
    expect = _host_mask(nx, ny, **kw)
    nat.check(nat.load().lbm_mask_add_obstacle(nx, ny, nat.ptr(expect), 120, 64))
    assert np.array_equal(sim.info().view(np.uint8), expect.view(np.uint8))
    sim.close()


def test_checkpoint_and_reset_after_device_scene(gpu, tmp_path):
    nx, ny = 192, 96
    kw = _kw("channel", 21, 0.05, (4.0, 9.0))
    a = FluidSimulator(nx, ny, **kw)
    a.step(50)
    path = str(tmp_path / "ck.bin")
    a.save(path)
    b = FluidSimulator(nx, ny, **kw)
    b.load(path)
    assert np.array_equal(a.read_populations(), b.read_populations())
    a.step(20)
    b.step(20)
    assert np.array_equal(a.read_populations(), b.read_populations())
    b.reset()
    assert np.array_equal(b.info().view(np.uint8), _host_mask(nx, ny, **kw).view(np.uint8))
    a.close()
    b.close()


def test_edits_after_reset_on_a_device_scene(gpu):
    """A reset rebuilds the scene on the device; the batched edits that follow start from the
    initial mask again (their device copy of the host mask is refreshed)."""
    nx, ny = 256, 128
    kw = _kw("channel", 13, 0.05, (4.0, 9.0))
    sim = FluidSimulator(nx, ny, **kw)
    sim.apply_edits([("obstacle", 60, 64)])
    sim.step(5)
    sim.reset()
    assert np.array_equal(sim.info().view(np.uint8), _host_mask(nx, ny, **kw).view(np.uint8))
    sim.apply_edits([("obstacle", 180, 64)])
    expect = _host_mask(nx, ny, **kw)
    nat.check(nat.load().lbm_mask_add_obstacle(nx, ny, nat.ptr(expect), 180, 64))
    assert np.array_equal(sim.info().view(np.uint8), expect.view(np.uint8))
    sim.close()
