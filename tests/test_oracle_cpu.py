"""The oracle itself: pinned to the golden fixtures of the independent pure-Python
restatement, and checked on analytic physics cases.  CPU only."""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_oracle_matches_golden(path):
    z = np.load(path)
    scene = str(z["scene"])
    ny, nx = z["info_in"].shape
    kw = {}
    if scene == "cavity":
        kw["lid_vx"] = float(z["speed"])
    if scene == "poiseuille":
        kw["inlet_vx"] = float(z["speed"])
    o = oracle.RefOracle(nx, ny, scene, tau=float(z["tau"]), **kw)
    assert np.array_equal(o.host_info, z["info_in"])  # lattice.rs mask
    o.info[...] = z["info_init"]
    for s in range(int(z["steps"])):
        if str(z["edit"]) == "obstacle" and s == 2:
            assert o.add_obstacle(32, 30) == 0
        o.step()
    assert np.array_equal(o.populations, z["pops"])
    assert np.array_equal(o.macro4, z["macro"])
    assert np.array_equal(o.info, z["info_out"])


def test_golden_fixtures_exist():
    assert len(FIXTURES) >= 4


def test_pyref_masks_match_oracle():
    import sys

    sys.path.insert(0, GOLDEN)
    import pyref

    for scene, nx, ny in (("poiseuille", 200, 120), ("cavity", 33, 21), ("custom", 9, 7), ("poiseuille", 600, 375)):
        assert np.array_equal(pyref.mask(nx, ny, scene), oracle.mask_reference(nx, ny, scene))


def test_physics_f64_mass_exact_in_closed_cavity():
    p = oracle.PhysOracle(oracle.mask_physics_cavity(64, 48, 0.1), 0.6, np.float64)
    m0 = p.conservation()[0]
    p.step(500)
    assert abs(p.conservation()[0] - m0) / m0 < 1e-13


def test_physics_f32_mass_drift_bounded():
    p = oracle.PhysOracle(oracle.mask_physics_cavity(128, 128, 0.1), 0.6, np.float32)
    m0 = p.conservation()[0]
    p.step(1000)
    assert abs(p.conservation()[0] - m0) / m0 < 1e-10


def test_rest_state_is_invariant():
    info = oracle.mask_physics_channel(128, 64, 0.0, 1, 0.05, 4.0, 8.0)[0]
    p = oracle.PhysOracle(info, 0.7, np.float64)
    p.step(50)
    assert np.max(np.abs(p.deviations)) < 1e-15


def _periodic_info(nx, ny):
    info = np.zeros((ny, nx), oracle.INFO_DTYPE)
    info["material"] = 1
    info["block_iter"] = -1
    return info


@pytest.mark.parametrize("collision", [0, 1, 2, 3], ids=["bgk", "regularized", "mrt", "kbc"])
def test_collisions_conserve_mass_and_momentum(collision):
    """Every collision operator of the oracle conserves mass and momentum (FP64, periodic
    lattice, a random non-equilibrium state)."""
    nx, ny = 48, 32
    p = oracle.PhysOracle(_periodic_info(nx, ny), 0.53, np.float64, collision=collision)
    rng = np.random.default_rng(collision)
    p.bufs[p.cur][...] = oracle.PhysOracle.W.reshape(9, 1, 1) * 0.05 * rng.standard_normal((9, ny, nx))
    before = np.array(p.conservation())
    p.step(20)
    after = np.array(p.conservation())
    assert np.all(np.isfinite(p.deviations))
    assert abs(after[0] - before[0]) <= 1e-12 * abs(before[0])
    assert np.max(np.abs(after[1:] - before[1:])) <= 1e-12 * abs(before[0])


@pytest.mark.parametrize("collision", [0, 1, 2, 3], ids=["bgk", "regularized", "mrt", "kbc"])
def test_uniform_flow_equilibrium_is_a_fixed_point(collision):
    nx, ny = 32, 16
    p = oracle.PhysOracle(_periodic_info(nx, ny), 0.6, np.float64, collision=collision)
    ux = np.full((ny, nx), 0.05)
    uy = np.full((ny, nx), -0.02)
    p.init_equilibrium(np.full((ny, nx), 1.01), ux, uy)
    f0 = p.populations().copy()
    p.step(10)
    assert np.max(np.abs(p.populations() - f0)) < 1e-13


def test_inlet_velocity_and_outlet_density_are_imposed():
    """The Zou-He inlet's cells carry exactly the prescribed parabolic velocity, and the anchored
    outflow keeps the outlet density at 1 (FP64)."""
    info, _ = oracle.mask_physics_channel(96, 34, 0.05, 1, 0.0, 4.0, 8.0)
    p = oracle.PhysOracle(info, 0.7, np.float64)
    p.step(300)
    rho, ux, uy = p.macro()
    inlet, outlet = info["material"] == 3, info["material"] == 5
    assert np.max(np.abs(ux[inlet] - info["vx"][inlet])) < 1e-15
    assert np.max(np.abs(uy[inlet])) < 1e-15
    assert np.max(np.abs(rho[outlet] - 1.0)) < 1e-14


def test_shear_wave_decay_rate():
    nx, ny, tau, U, steps = 32, 128, 0.8, 0.01, 2000
    p = oracle.PhysOracle(oracle.mask_periodic(nx, ny), tau, np.float64)
    y = np.arange(ny)
    p.init_equilibrium(None, np.tile((U * np.sin(2 * np.pi * y / ny))[:, None], (1, nx)), None)
    p.step(steps)
    _, ux, _ = p.macro()
    amp = 2.0 * np.mean(ux * np.sin(2 * np.pi * y / ny)[:, None])
    expected = U * np.exp(-(tau - 0.5) / 3.0 * (2 * np.pi / ny) ** 2 * steps)
    assert abs(amp - expected) / expected < 2e-3


def test_poiseuille_channel_profile():
    """Empty channel: the Zou-He parabolic inlet profile is carried to the outlet."""
    nx, ny = 96, 34
    info, nd = oracle.mask_physics_channel(nx, ny, 0.04, 1, 0.0, 8.0, 8.0)
    assert nd == 0
    p = oracle.PhysOracle(info, 0.8, np.float64)
    p.step(6000)
    _, ux, _ = p.macro()
    H = ny - 2
    s = np.arange(1, ny - 1) - 0.5
    expected = 4 * 0.04 * s * (H - s) / H**2
    prof = ux[1:-1, nx // 2]
    assert np.max(np.abs(prof - expected)) / 0.04 < 0.02


def test_channel_mask_properties():
    nx, ny = 1024, 512
    a, nd = oracle.mask_physics_channel(nx, ny, 0.05, 42, 0.05, 8.0, 32.0)
    b, nd2 = oracle.mask_physics_channel(nx, ny, 0.05, 42, 0.05, 8.0, 32.0)
    c, _ = oracle.mask_physics_channel(nx, ny, 0.05, 43, 0.05, 8.0, 32.0)
    assert nd == nd2 and np.array_equal(a, b)
    assert not np.array_equal(a, c)
    frac = (a["material"] == 4).mean()
    assert 0.05 <= frac < 0.06
    assert (a["material"][:, 0] == 3)[1:-1].all() and (a["material"][:, -1] == 5)[1:-1].all()
    assert (a["material"][0] == 2).all() and (a["material"][-1] == 2).all()


def test_closure_oracle_backprop_matches_finite_differences():
    from oracle import closure_ref as ref

    rng = np.random.default_rng(0)
    n = 9 * 9 * 32 + 32 + 9 * 32 * 32 + 32 + 9 * 32 * 9 + 9
    p = rng.standard_normal(n) * 0.1
    x0 = rng.standard_normal((1, 12, 12, 9))
    T = 0.3 * rng.standard_normal((1, 12, 12, 9))
    _, g = ref.loss_and_grad(x0, T, p, emulate_bf16=False)
    for i in rng.choice(n, 12, replace=False):
        e = np.zeros(n)
        e[i] = 1e-6
        fd = (ref.loss_and_grad(x0, T, p + e, False)[0] - ref.loss_and_grad(x0, T, p - e, False)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-5 * (abs(fd) + abs(g[i])) + 1e-12


def test_closure_projection_conserves_moments():
    from oracle import closure_ref as ref

    v = np.random.default_rng(1).standard_normal((50, 9))
    pv = ref.project(v)
    assert np.max(np.abs(pv.sum(-1))) < 1e-12
    assert np.max(np.abs((pv * ref.EX).sum(-1))) < 1e-12 and np.max(np.abs((pv * ref.EY).sum(-1))) < 1e-12
    # the transpose really is the adjoint
    g = np.random.default_rng(2).standard_normal((50, 9))
    assert abs((ref.project(v) * g).sum() - (v * ref.project_t(g)).sum()) < 1e-10


def test_closure_stress_loss_gradient_against_finite_differences():
    """The restatement of the stress target's loss: its gradient against central differences."""
    from oracle import closure_ref as ref

    rng = np.random.default_rng(0)
    p = 0.05 * rng.standard_normal(9 * 9 * 32 + 32 + 9 * 32 * 32 + 32 + 9 * 32 * 9 + 9)
    x0 = rng.standard_normal((1, 16, 16, 9))
    T = 0.1 * rng.standard_normal((1, 16, 16, 9))
    _, g = ref.stress_loss_and_grad(x0, T, p, 0.7, emulate_bf16=False)
    for k in (5, 2600, 3000, 9000, 12000, 14468):
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += e
        pm[k] -= e
        fd = (ref.stress_loss_and_grad(x0, T, pp, 0.7, False)[0] - ref.stress_loss_and_grad(x0, T, pm, 0.7, False)[0]) / (2 * e)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, (k, fd, g[k])
