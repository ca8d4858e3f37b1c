"""Physics-mode parity (exact weights, half-way bounce-back, moving lid, Zou-He inlet,
zero-gradient outflow) of the CUDA step against the oracle, plus analytic checks.

Tolerances: FP32 max relative error <= 1e-5 on rho and u after one step (velocity
normalised by the lid / inlet speed) and relative L2 <= 1e-4 after 1000 steps; FP64
<= 1e-12; FP32 mass drift <= 1e-10 relative over 1000 steps of a closed cavity.
"""
import numpy as np
import pytest

import oracle
from conftest import rel_l2
from simuverse_gb300 import FluidSimulator

pytestmark = pytest.mark.gpu


def _macro_err(sim, ref, u_scale):
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    e_rho = float(np.max(np.abs(rho - r_rho)))
    e_u = float(max(np.max(np.abs(ux - r_ux)), np.max(np.abs(uy - r_uy)))) / u_scale
    return e_rho, e_u


def test_cavity_fp32_parity_and_mass(gpu):
    nx = ny = 256
    sim = FluidSimulator(nx, ny, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)
    info = oracle.mask_physics_cavity(nx, ny, 0.1)
    assert np.array_equal(sim.info(), info)
    ref = oracle.PhysOracle(info, 0.6, np.float32)
    m0 = sim.conservation()[0]
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, 0.1)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    sim.step(999)
    ref.step(999)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4
    m1 = sim.conservation()[0]
    assert abs(m1 - m0) / m0 <= 1e-10
    mo = ref.conservation()[0]
    assert abs(m1 - mo) / mo <= 1e-10


def test_cavity_fp64_parity(gpu):
    nx, ny = 96, 80
    sim = FluidSimulator(nx, ny, mode="physics", dtype="f64", scene="cavity", tau=0.55, lid_speed=0.08)
    ref = oracle.PhysOracle(oracle.mask_physics_cavity(nx, ny, 0.08), 0.55, np.float64)
    sim.step(300)
    ref.step(300)
    e_rho, e_u = _macro_err(sim, ref, 0.08)
    assert e_rho <= 1e-6 and e_u <= 1e-6  # macro planes are FP32
    f = sim.read_populations(np.float64)
    assert np.max(np.abs(f - ref.populations(np.float64))) <= 1e-12
    m_sim, m_ref = sim.conservation()[0], ref.conservation()[0]
    assert abs(m_sim - m_ref) / m_ref <= 1e-13


def test_channel_fp32_parity(gpu):
    nx, ny = 384, 160
    kw = dict(inlet_speed=0.05, seed=11, solid_fraction=0.05, disk_radius=(5.0, 12.0))
    sim = FluidSimulator(nx, ny, mode="physics", scene="channel", tau=0.56, **kw)
    info, ndisk = oracle.mask_physics_channel(nx, ny, 0.05, 11, 0.05, 5.0, 12.0)
    assert ndisk > 3
    assert np.array_equal(sim.info(), info)
    ref = oracle.PhysOracle(info, 0.56, np.float32)
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, 0.05)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    sim.step(999)
    ref.step(999)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4


@pytest.mark.parametrize("scene,nx,ny", [("cavity", 65535, 5), ("cavity", 5, 65535), ("channel", 65535, 40),
                                         ("channel", 40, 20000)])
def test_extreme_aspect_parity(gpu, scene, nx, ny):
    """The largest side the lattice takes (65535) as a row and as a column, a lattice whose rows
    are longer than any block and one whose grid is all rows: 1 step at the 1e-5 bar, 60 steps
    at the 1e-4 L2 bar."""
    if scene == "cavity":
        sim = FluidSimulator(nx, ny, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)
        info = oracle.mask_physics_cavity(nx, ny, 0.1)
        u_scale = 0.1
    else:
        sim = FluidSimulator(nx, ny, mode="physics", scene="channel", tau=0.56, inlet_speed=0.05, seed=5,
                             solid_fraction=0.05, disk_radius=(3.0, 6.0))
        info, _ = oracle.mask_physics_channel(nx, ny, 0.05, 5, 0.05, 3.0, 6.0)
        u_scale = 0.05
    assert np.array_equal(sim.info(), info)
    ref = oracle.PhysOracle(info, sim.tau, np.float32)
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, u_scale)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    sim.step(59)
    ref.step(59)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4
    sim.close()


def test_channel_4096_10000_steps_against_fp64(gpu):
    """The C2 configuration for its full 10,000 steps (4096² channel, tau 0.56, seed 1234), FP32 and
    FP16 with stochastic rounding against an FP64 run of the same lattice: no non-finite
    population, and the relative L2 errors of rho and u and the mass (open channel: inflow minus
    outflow) within the stated bounds, about 3x the measured 8.5e-6 / 1.8e-4 / 7.5e-6 (FP32) and
    4.3e-5 / 8.5e-4 / 9.5e-6 (FP16)."""
    kw = dict(mode="physics", scene="channel", tau=0.56, inlet_speed=0.05, solid_fraction=0.05,
              disk_radius=(8.0, 32.0), seed=1234)
    ref = FluidSimulator(4096, 4096, dtype="f64", **kw)
    sims = {"f32": FluidSimulator(4096, 4096, dtype="f32", **kw),
            "f16": FluidSimulator(4096, 4096, dtype="f16", rounding="stochastic", **kw)}
    bounds = {"f32": (3e-5, 6e-4, 3e-5), "f16": (1.5e-4, 2.5e-3, 3e-5)}
    for _ in range(10):
        ref.step(1000)
        for s in sims.values():
            s.step(1000)
    m_ref = ref.conservation()[0]
    for k, s in sims.items():
        e_rho, e_u, _, _ = s.macro_error(ref)
        assert s.nonfinite_count() == 0
        b_rho, b_u, b_m = bounds[k]
        assert e_rho <= b_rho and e_u <= b_u, (k, e_rho, e_u)
        assert abs(s.conservation()[0] - m_ref) / m_ref <= b_m
        s.close()
    ref.close()


def test_shear_wave_decay_matches_viscosity(gpu):
    """Periodic shear wave u_x = U sin(2 pi y / ny) decays as exp(-nu k^2 t), nu = (tau - 1/2)/3."""
    nx, ny, tau, U, steps = 64, 128, 0.8, 0.01, 2000
    sim = FluidSimulator(nx, ny, mode="physics", dtype="f64", scene="periodic", tau=tau)
    y = np.arange(ny)
    ux = np.tile((U * np.sin(2 * np.pi * y / ny))[:, None], (1, nx))
    sim.init_equilibrium(None, ux, None)
    sim.step(steps)
    _, ux1, _ = sim.read_macro()
    amp = 2.0 * np.mean(ux1 * np.sin(2 * np.pi * y / ny)[:, None])
    nu = (tau - 0.5) / 3.0
    k = 2 * np.pi / ny
    expected = U * np.exp(-nu * k * k * steps)
    assert abs(amp - expected) / expected < 5e-3


def test_precision_forms_against_fp64(gpu):
    nx, ny = 256, 128
    kw = dict(mode="physics", scene="channel", tau=0.6, inlet_speed=0.05, seed=3, disk_radius=(5.0, 10.0))
    ref = FluidSimulator(nx, ny, dtype="f64", **kw)
    ref.step(2000)
    errs = {}
    for dt in ("f32", "f16", "bf16"):
        s = FluidSimulator(nx, ny, dtype=dt, **kw)
        s.step(2000)
        errs[dt] = s.macro_error(ref)
        assert s.nonfinite_count() == 0
    print("rel L2 (rho, u) and max |du|, |drho| against FP64:", errs)
    assert errs["f32"][1] < 5e-5
    assert errs["f16"][1] < 1e-3
    assert errs["bf16"][1] < 2e-2


def test_init_equilibrium_roundtrip(gpu):
    nx, ny = 80, 60
    rng = np.random.default_rng(5)
    rho = (1.0 + 0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
    ux = (0.03 * rng.standard_normal((ny, nx))).astype(np.float32)
    uy = (0.03 * rng.standard_normal((ny, nx))).astype(np.float32)
    sim = FluidSimulator(nx, ny, mode="physics", scene="periodic", tau=0.7)
    sim.init_equilibrium(rho, ux, uy)
    f = sim.read_populations(np.float64)
    ex = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])[:, None, None]
    ey = np.array([0, 0, -1, 0, 1, -1, -1, 1, 1])[:, None, None]
    r = f.sum(0)
    assert np.max(np.abs(r - rho)) < 1e-6
    assert np.max(np.abs((ex * f).sum(0) / r - ux)) < 1e-6
    assert np.max(np.abs((ey * f).sum(0) / r - uy)) < 1e-6


@pytest.mark.parametrize("scene,nx,ny", [("channel", 388, 150), ("cavity", 132, 100), ("periodic", 68, 36),
                                         ("channel", 1024, 96)])
@pytest.mark.parametrize("dtype", ["f32", "f64", "f16", "bf16"])
@pytest.mark.parametrize("kernel", ["vec4", "vec2"])
def test_vec_kernels_match_cell_kernel(gpu, scene, nx, ny, dtype, kernel):
    """The two- and four-cells-per-thread kernels agree with the one-cell kernel."""
    kw = dict(mode="physics", dtype=dtype, scene=scene, tau=0.58, lid_speed=0.1, inlet_speed=0.05, seed=5,
              disk_radius=(4.0, 9.0))
    a = FluidSimulator(nx, ny, kernel=kernel, **kw)
    b = FluidSimulator(nx, ny, kernel="cell", **kw)
    if scene == "periodic":
        rng = np.random.default_rng(2)
        u = (0.02 * rng.standard_normal((2, ny, nx))).astype(np.float32)
        a.init_equilibrium(None, u[0], u[1])
        b.init_equilibrium(None, u[0], u[1])
    a.step(200)
    b.step(200)
    fa, fb = a.read_populations(np.float64), b.read_populations(np.float64)
    fluid = ~np.isin(a.info()["material"], (2, 4))
    tol = {"f32": 1e-6, "f64": 1e-13, "f16": 5e-4, "bf16": 5e-3}[dtype]
    assert np.max(np.abs(fa - fb)[:, fluid]) <= tol
    for x, y in zip(a.read_macro(), b.read_macro()):
        assert np.max(np.abs(x - y)[fluid]) <= 10 * tol


def test_vec4_channel_parity_with_oracle(gpu):
    nx, ny = 516, 130
    info, _ = oracle.mask_physics_channel(nx, ny, 0.05, 9, 0.05, 4.0, 10.0)
    sim = FluidSimulator(nx, ny, mode="physics", scene="channel", tau=0.56, inlet_speed=0.05, seed=9,
                         disk_radius=(4.0, 10.0), kernel="vec4")
    ref = oracle.PhysOracle(info, 0.56, np.float32)
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, 0.05)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    sim.step(499)
    ref.step(499)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4


@pytest.mark.parametrize("scene,nx,ny", [("channel", 392, 150), ("cavity", 136, 100), ("periodic", 72, 36),
                                         ("channel", 1032, 66), ("periodic", 520, 20)])
@pytest.mark.parametrize("dtype", ["f32", "f64", "f16", "bf16"])
def test_bulk_kernel_matches_cell_kernel(gpu, scene, nx, ny, dtype):
    """The bulk-copy fed kernel agrees with the one-cell kernel, including partial tiles
    and the periodic wrap at both row ends."""
    kw = dict(mode="physics", dtype=dtype, scene=scene, tau=0.58, lid_speed=0.1, inlet_speed=0.05, seed=5,
              disk_radius=(4.0, 9.0))
    a = FluidSimulator(nx, ny, kernel="bulk", **kw)
    b = FluidSimulator(nx, ny, kernel="cell", **kw)
    if scene == "periodic":
        rng = np.random.default_rng(2)
        u = (0.02 * rng.standard_normal((2, ny, nx))).astype(np.float32)
        a.init_equilibrium(None, u[0], u[1])
        b.init_equilibrium(None, u[0], u[1])
    a.step(150)
    b.step(150)
    a.status()
    fa, fb = a.read_populations(np.float64), b.read_populations(np.float64)
    fluid = ~np.isin(a.info()["material"], (2, 4))
    tol = {"f32": 1e-6, "f64": 1e-13, "f16": 5e-4, "bf16": 5e-3}[dtype]
    assert np.max(np.abs(fa - fb)[:, fluid]) <= tol
    for x, y in zip(a.read_macro(), b.read_macro()):
        assert np.max(np.abs(x - y)[fluid]) <= 10 * tol


@pytest.mark.parametrize("collision", ["regularized", "mrt", "kbc"])
def test_collision_variants_match_oracle(gpu, collision):
    nx, ny = 96, 80
    code = {"regularized": 1, "mrt": 2, "kbc": 3}[collision]
    sim = FluidSimulator(nx, ny, mode="physics", scene="cavity", tau=0.55, lid_speed=0.08, collision=collision)
    ref = oracle.PhysOracle(oracle.mask_physics_cavity(nx, ny, 0.08), 0.55, np.float32, collision=code)
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, 0.08)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    m0 = sim.conservation()[0]
    sim.step(499)
    ref.step(499)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4
    assert abs(sim.conservation()[0] - m0) / m0 <= 1e-10


def test_read_macro_into_caller_buffers(gpu):
    torch = pytest.importorskip("torch")
    sim = FluidSimulator(128, 64, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)
    sim.step(30)
    ref = sim.read_macro()
    pinned = torch.empty((3, 64, 128), dtype=torch.float32, pin_memory=True).numpy()
    got = sim.read_macro(out=(pinned[0], pinned[1], pinned[2]))
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    with pytest.raises(ValueError):
        sim.read_macro(out=(np.empty(5, np.float32),) * 3)


def test_kbc_decaying_turbulence_matches_oracle(gpu):
    """KBC at tau 0.5005 on a periodic decaying-turbulence field (the collision and the
    regime of the learned-closure study): max relative error <= 1e-5 (velocity relative to
    u_rms) after one step, relative L2 <= 1e-4 after 300 steps; mass kept to 1e-10 relative
    (the rest population closes the mass balance), momentum to FP32 rounding: a drift of the
    total below 1e-8 of the total mass, and within that of the oracle's."""
    from simuverse_gb300.turbulence import random_velocity

    n = 256
    ux, uy = random_velocity(n, 4242, k0=8.0, u_rms=0.04)
    ux, uy = ux.astype(np.float32), uy.astype(np.float32)
    sim = FluidSimulator(n, n, mode="physics", scene="periodic", tau=0.5005, collision="kbc")
    sim.init_equilibrium(None, ux, uy)
    ref = oracle.PhysOracle(oracle.mask_periodic(n, n), 0.5005, np.float32, collision=3)
    ref.init_equilibrium(None, ux, uy)
    c0 = sim.conservation()
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, 0.04)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    sim.step(299)
    ref.step(299)
    rho, ux1, uy1 = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux1, uy1]), np.stack([r_ux, r_uy])) <= 1e-4
    c1 = sim.conservation()
    assert abs(c1[0] - c0[0]) / c0[0] <= 1e-10
    assert abs(c1[1] - c0[1]) <= 1e-8 * c0[0] and abs(c1[2] - c0[2]) <= 1e-8 * c0[0]
    co = ref.conservation()
    assert abs(c1[1] - co[1]) <= 1e-8 * c0[0] and abs(c1[2] - co[2]) <= 1e-8 * c0[0]


def test_channel_4096_parity_with_oracle(gpu):
    """The benchmarked workload at full size: channel 4096^2, Zou-He inlet u = 0.05, outflow,
    walls, disks r 8-32 at 5 % solid, seed 1234, tau 0.56.  Same mask as the oracle's, max
    relative error <= 1e-5 after one step, relative L2 <= 1e-4 after 200 steps."""
    n = 4096
    kw = dict(inlet_speed=0.05, seed=1234, solid_fraction=0.05, disk_radius=(8.0, 32.0))
    sim = FluidSimulator(n, n, mode="physics", scene="channel", tau=0.56, **kw)
    info, ndisk = oracle.mask_physics_channel(n, n, 0.05, 1234, 0.05, 8.0, 32.0)
    assert ndisk > 100
    assert np.array_equal(sim.info(), info)
    ref = oracle.PhysOracle(info, 0.56, np.float32)
    sim.step(1)
    ref.step(1)
    e_rho, e_u = _macro_err(sim, ref, 0.05)
    assert e_rho <= 1e-5 and e_u <= 1e-5
    sim.step(199)
    ref.step(199)
    rho, ux, uy = sim.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4
    sim.close()


def test_bulk_kernel_handles_on_two_devices(gpu):
    """The bulk-copy kernel's shared-memory attribute and grid size are set up per device: an
    FP64 handle (about 76 KB of dynamic shared memory) steps on every visible device."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU visible")
    prev = torch.cuda.current_device()
    results = []
    try:
        for dev in (0, 1):
            torch.cuda.set_device(dev)
            s = FluidSimulator(136, 100, mode="physics", dtype="f64", scene="cavity", tau=0.58, lid_speed=0.1,
                               kernel="bulk")
            s.step(20)
            s.status()
            results.append(s.read_populations(np.float64))
            s.close()
    finally:
        torch.cuda.set_device(prev)
    assert np.array_equal(results[0], results[1])
