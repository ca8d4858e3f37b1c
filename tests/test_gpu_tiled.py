"""The tiled 16-bit population layout (LBM_KERNEL_TILED, the default for FP16 / BF16 when
nx % 64 == 0): same results as the two-cell kernel over the SoA layout, layout-independent
read-back and write, conservation sums, and checkpoints that refuse the other layout."""
import numpy as np
import pytest

from simuverse_gb300 import FluidSimulator

pytestmark = pytest.mark.gpu

CASES = [("channel", 256, 96), ("cavity", 128, 64), ("periodic", 192, 128)]


def _pair(scene, nx, ny, dtype):
    kw = dict(mode="physics", dtype=dtype, scene=scene, tau=0.58, lid_speed=0.1, inlet_speed=0.05, seed=5,
              disk_radius=(4.0, 9.0))
    a = FluidSimulator(nx, ny, kernel="tiled", **kw)
    b = FluidSimulator(nx, ny, kernel="vec2", **kw)
    if scene == "periodic":
        rng = np.random.default_rng(2)
        u = (0.02 * rng.standard_normal((2, ny, nx))).astype(np.float32)
        a.init_equilibrium(None, u[0], u[1])
        b.init_equilibrium(None, u[0], u[1])
    return a, b


@pytest.mark.parametrize("dtype", ["f16", "bf16"])
@pytest.mark.parametrize("scene,nx,ny", CASES)
def test_tiled_matches_soa_two_cell_kernel(gpu, scene, nx, ny, dtype):
    a, b = _pair(scene, nx, ny, dtype)
    assert np.array_equal(a.read_populations(), b.read_populations())  # the same initial state
    a.step(150)
    b.step(150)
    fa, fb = a.read_populations(np.float64), b.read_populations(np.float64)
    fluid = ~np.isin(a.info()["material"], (2, 4))
    tol = {"f16": 5e-4, "bf16": 5e-3}[dtype]
    assert np.max(np.abs(fa - fb)[:, fluid]) <= tol
    for x, y in zip(a.read_macro(), b.read_macro()):
        assert np.max(np.abs(x - y)[fluid]) <= 10 * tol
    ca, cb = np.array(a.conservation()), np.array(b.conservation())
    assert np.max(np.abs(ca - cb)) <= 1e-3 * abs(cb[0])
    a.close()
    b.close()


def test_tiled_write_read_round_trip(gpu):
    nx, ny = 128, 64
    sim = FluidSimulator(nx, ny, mode="physics", dtype="f16", scene="periodic", tau=0.7, kernel="tiled")
    rng = np.random.default_rng(4)
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)[:, None, None]
    f = (w * (1.0 + 0.01 * rng.standard_normal((9, ny, nx)))).astype(np.float32)
    sim.write_populations(f)
    back = sim.read_populations()
    assert np.max(np.abs(back - f)) < 2e-5  # FP16 rounding of (f - w) * 2^10
    # one step equals the SoA kernel's step from the same populations
    ref = FluidSimulator(nx, ny, mode="physics", dtype="f16", scene="periodic", tau=0.7, kernel="vec2")
    ref.write_populations(f)
    sim.step(1)
    ref.step(1)
    assert np.max(np.abs(sim.read_populations() - ref.read_populations())) < 1e-6
    sim.close()
    ref.close()


def test_tiled_checkpoint_refuses_other_layout(gpu, tmp_path):
    kw = dict(mode="physics", dtype="bf16", scene="cavity", tau=0.6, lid_speed=0.1)
    a = FluidSimulator(128, 64, kernel="tiled", **kw)
    a.step(10)
    path = str(tmp_path / "t.ckpt")
    a.save(path)
    b = FluidSimulator(128, 64, kernel="tiled", **kw)
    b.load(path)
    assert np.array_equal(a.read_populations(), b.read_populations())
    c = FluidSimulator(128, 64, kernel="vec2", **kw)
    with pytest.raises(Exception):
        c.load(path)
    for s in (a, b, c):
        s.close()


def test_tiled_rejected_where_it_does_not_apply(gpu):
    with pytest.raises(Exception):
        FluidSimulator(100, 64, mode="physics", dtype="f16", scene="cavity", kernel="tiled")  # nx % 64
    with pytest.raises(Exception):
        FluidSimulator(128, 64, mode="physics", dtype="f32", scene="cavity", kernel="tiled")  # FP32


# LBM_KERNEL_RING: the tiled kernel's rules with the rows staged in shared memory by bulk copies.
# Strips of 8 tiles, so 576 = 9 tiles leaves a one-tile strip, 64 is a lattice of one tile, and
# 4 or 5 rows wrap inside one block's row range.
RING_CASES = [("channel", 576, 37), ("channel", 1024, 300), ("cavity", 128, 64), ("periodic", 512, 4),
              ("periodic", 64, 5), ("periodic", 192, 7)]


def _bits(sim):
    return sim.read_populations().view(np.uint32)


@pytest.mark.parametrize("rounding", ["nearest", "stochastic"])
@pytest.mark.parametrize("dtype", ["f16", "bf16"])
@pytest.mark.parametrize("scene,nx,ny", RING_CASES)
def test_ring_matches_tiled_bit_for_bit(gpu, scene, nx, ny, dtype, rounding):
    kw = dict(mode="physics", dtype=dtype, scene=scene, tau=0.58, lid_speed=0.1, inlet_speed=0.05, seed=5,
              disk_radius=(4.0, 9.0), rounding=rounding)
    a = FluidSimulator(nx, ny, kernel="ring", **kw)
    b = FluidSimulator(nx, ny, kernel="tiled", **kw)
    if scene == "periodic":
        rng = np.random.default_rng(3)
        u = (0.02 * rng.standard_normal((2, ny, nx))).astype(np.float32)
        a.init_equilibrium(None, u[0], u[1])
        b.init_equilibrium(None, u[0], u[1])
    a.step(37)
    b.step(37)
    if scene == "channel":  # a force stroke and an obstacle: forcing cells and new walls mid-run
        for s in (a, b):
            s.add_external_force((nx * 0.4, ny * 0.5), (nx * 0.35, ny * 0.45))
            if ny >= 64:  # the obstacle is a disc of radius 28
                s.add_obstacle(nx // 2, ny // 2)
    a.step(40)
    b.step(40)
    a.status()
    assert np.array_equal(_bits(a), _bits(b))
    for x, y in zip(a.read_macro(), b.read_macro()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    a.close()
    b.close()


@pytest.mark.parametrize("dtype", ["f16", "bf16"])
def test_ring_macro_every_step_and_full_size(gpu, dtype):
    """The macro-writing form, and the 4096^2 channel (one wave of blocks, 8 strips)."""
    for nx, ny, steps in ((640, 200, 25), (4096, 4096, 6)):
        kw = dict(mode="physics", dtype=dtype, scene="channel", tau=0.56, inlet_speed=0.05, seed=11,
                  macro_every_step=True)
        a = FluidSimulator(nx, ny, kernel="ring", **kw)
        b = FluidSimulator(nx, ny, kernel="tiled", **kw)
        a.step(steps)
        b.step(steps)
        a.status()
        assert np.array_equal(_bits(a), _bits(b))
        for x, y in zip(a.read_macro(), b.read_macro()):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
        a.close()
        b.close()


def test_ring_checkpoint_shares_the_tiled_layout(gpu, tmp_path):
    kw = dict(mode="physics", dtype="f16", scene="cavity", tau=0.6, lid_speed=0.1)
    a = FluidSimulator(128, 64, kernel="ring", **kw)
    a.step(10)
    path = str(tmp_path / "r.ckpt")
    a.save(path)
    b = FluidSimulator(128, 64, kernel="tiled", **kw)
    b.load(path)
    a.step(5)
    b.step(5)
    assert np.array_equal(_bits(a), _bits(b))
    a.close()
    b.close()
    with pytest.raises(Exception):
        FluidSimulator(100, 64, mode="physics", dtype="f16", scene="cavity", kernel="ring")  # nx % 64
    with pytest.raises(Exception):
        FluidSimulator(128, 64, mode="physics", dtype="f32", scene="cavity", kernel="ring")  # FP32
