"""Consumers of the macro field on the GPU against the oracle: particle advection and the
splat canvas (bit for bit; deterministic splats = the oracle's ascending order), the
canvas presentation, the curl field (bit for bit) and the field colour maps (to rounding:
atan2 and the filtering order are the only non-exact steps)."""
import numpy as np
import pytest

import oracle
from simuverse_gb300 import FluidSimulator
from simuverse_gb300.view import Particles, colorize, curl

pytestmark = pytest.mark.gpu


def _sim(kind):
    if kind == "poiseuille":  # reference mode, the reference UI's scene (fluid_ty 0)
        return FluidSimulator(200, 120, mode="reference", scene="poiseuille", tau=0.56)
    return FluidSimulator(96, 64, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)  # fluid_ty 1


@pytest.mark.parametrize("kind", ["poiseuille", "cavity"])
@pytest.mark.parametrize("point", [1, 2, 5])
def test_particles_match_oracle(gpu, kind, point):
    sim = _sim(kind)
    ps = Particles(sim, count=2500, life_time=9.0, point_size=point, seed=4)
    st = ps.state()
    cw, ch = ps.canvas_w, ps.canvas_h
    canvas = np.zeros((ch, cw, 3), np.float32)
    pois = kind == "poiseuille"
    # before the first step the field is zero: particles age but do not move
    ps.update()
    oracle.particles_update(np.zeros((sim.ny, sim.nx), np.float32), np.zeros((sim.ny, sim.nx), np.float32), True,
                            sim.pixel_size, 9.0, 4.15, point, cw, ch, pois, st, canvas)
    assert np.array_equal(ps.state(), st)
    for it in range(24):
        sim.step(1)
        ps.update()
        _, ux, uy = sim.read_macro()
        oracle.particles_update(ux, uy, False, sim.pixel_size, 9.0, 4.15, point, cw, ch, pois, st, canvas)
        got = ps.state()
        assert np.array_equal(got, st), (it, np.argwhere(got != st)[:5])
        assert np.array_equal(ps.canvas(), canvas), it
    assert np.count_nonzero(canvas[..., 0]) > 0
    moved = np.abs(st[:, :2] - st[:, 2:4]).max()
    assert moved > 0.5
    ps.close()
    sim.close()


@pytest.mark.parametrize("color_ty", [0, 1, 2])
def test_present_matches_oracle(gpu, color_ty):
    sim = _sim("poiseuille")
    ps = Particles(sim, count=3000, life_time=30.0, point_size=2, seed=1, color_ty=color_ty,
                   color=(0.2, 0.4, 0.6, 1.0))
    for _ in range(6):
        ps.compute()
    canvas = ps.canvas()
    for frame in range(3):
        ps.present()
        rgba_ref = oracle.present_canvas(canvas, color_ty, 1, 0.96, (0.2, 0.4, 0.6))
        got = ps.rgba()
        assert np.array_equal(ps.canvas(), canvas), frame  # the fade is exact
        assert np.array_equal(got[..., 3], rgba_ref[..., 3])
        assert np.max(np.abs(got - rgba_ref)) < 2e-6, (frame, np.max(np.abs(got - rgba_ref)))
    assert np.count_nonzero(rgba_ref[..., 3]) > 100
    ps.close()
    sim.close()


def test_fast_mode_positions_and_single_writer_pixels(gpu):
    sim = _sim("poiseuille")
    det = Particles(sim, count=4000, life_time=20.0, point_size=3, seed=9)
    fast = Particles(sim, count=4000, life_time=20.0, point_size=3, seed=9, deterministic=0)
    for _ in range(10):
        sim.step(1)
        det.update()
        fast.update()
    assert np.array_equal(det.state(), fast.state())
    a, b = det.canvas(), fast.canvas()
    assert np.array_equal(a[..., 0] > 0, b[..., 0] > 0)  # the same pixels are covered
    same = np.all(a == b, axis=-1)
    assert same.mean() > 0.9  # conflicts only where splats overlap
    for p in (det, fast):
        p.close()
    sim.close()


@pytest.mark.parametrize("kind", ["poiseuille", "cavity"])
def test_curl_matches_oracle(gpu, kind):
    sim = _sim(kind)
    zero = curl(sim)
    assert np.array_equal(zero, oracle.curl(np.zeros((sim.ny, sim.nx), np.float32),
                                            np.zeros((sim.ny, sim.nx), np.float32), True))
    sim.step(40)
    _, ux, uy = sim.read_macro()
    got = curl(sim)
    ref = oracle.curl(ux, uy)
    assert np.array_equal(got, ref), np.max(np.abs(got - ref))
    assert np.ptp(ref) > 0


@pytest.mark.parametrize("mode", ["curl", "angle"])
def test_colorize_matches_oracle(gpu, mode):
    sim = _sim("cavity")
    sim.step(60)
    rho, ux, uy = sim.read_macro()
    c = oracle.curl(ux, uy)
    # 2x (the UI's canvas), enlarged and reduced ragged canvases (pixel rows that share texel rows,
    # skip them, or fall in a partial block of 8 rows)
    for cw, ch in ((sim.nx * 2, sim.ny * 2), (sim.nx * 3 + 1, sim.ny - 5), (sim.nx // 2 + 3, sim.ny * 5 + 3),
                   (129, 7)):
        got = colorize(sim, mode, cw, ch)
        ref = oracle.colorize(rho, ux, uy, c if mode == "curl" else None, cw, ch, 0 if mode == "curl" else 1)
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) < 1e-5, np.max(np.abs(got - ref))
    sim.close()


def test_colorize_before_the_first_step(gpu):
    """Before the first step macro_tex holds zeros: the colour map samples a zero field."""
    sim = _sim("cavity")
    rho, ux, uy = sim.read_macro()
    c = curl(sim)
    for mode in ("curl", "angle"):
        got = colorize(sim, mode, 50, 30)
        ref = oracle.colorize(rho, ux, uy, c if mode == "curl" else None, 50, 30, 0 if mode == "curl" else 1, zero=True)
        assert np.max(np.abs(got - ref)) < 1e-5, (mode, np.max(np.abs(got - ref)))
    sim.close()


def test_curl_scalar_path_matches_oracle(gpu):
    """nx % 4 != 0 takes the one-cell curl kernel."""
    sim = FluidSimulator(98, 50, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)
    sim.step(30)
    _, ux, uy = sim.read_macro()
    assert np.array_equal(curl(sim), oracle.curl(ux, uy))
    sim.close()
