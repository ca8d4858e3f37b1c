"""Batched form: every method and tile form agrees with single-lattice runs of the same domains; the
persistent kernel's bounded grid barrier reports a missing arrival as LBM_ERR_TIMEOUT
and leaves the context usable; the autotuner returns a working configuration."""
import numpy as np
import pytest

from simuverse_gb300 import BatchSimulator, FluidSimulator, generate_domains
from simuverse_gb300 import _native as nat

pytestmark = pytest.mark.gpu

DOMAINS = [
    dict(nx=70, ny=45, scene="cavity", tau=0.6, speed=0.08),
    dict(nx=33, ny=97, scene="channel", tau=0.7, speed=0.05),
    dict(nx=128, ny=64, scene="channel", tau=0.56, speed=0.03),
    dict(nx=257, ny=130, scene="cavity", tau=0.9, speed=0.1),
    dict(nx=64, ny=64, scene="cavity", tau=0.55, speed=0.02),
    dict(nx=517, ny=66, scene="channel", tau=0.8, speed=0.07),
]


def _single(d, steps):
    sim = FluidSimulator(d["nx"], d["ny"], mode="physics", scene=d["scene"], tau=d["tau"], lid_speed=d["speed"],
                         inlet_speed=d["speed"], solid_fraction=0.0, kernel="cell")
    sim.step(steps)
    return sim


FORMS = {
    "rows": dict(cells_per_thread=1, linear=False, tile_threads_x=128, tile_rows=2, full_occupancy=False),
    "rows32": dict(cells_per_thread=1, linear=False, tile_threads_x=64, tile_rows=4, full_occupancy=True),
    "linear": dict(cells_per_thread=1, linear=True, tile_threads_x=64, tile_rows=2, full_occupancy=False),
    "linear32": dict(cells_per_thread=1, linear=True, tile_threads_x=256, tile_rows=1, full_occupancy=True),
    "vector4": dict(cells_per_thread=4, linear=False, tile_threads_x=32, tile_rows=4, full_occupancy=False),
}


@pytest.mark.parametrize("method,form", [("persistent", "rows"), ("persistent", "rows32"), ("persistent", "linear"),
                                         ("persistent", "linear32"), ("persistent", "vector4"),
                                         ("tile_launches", "linear"), ("tile_launches", "rows32"),
                                         ("domain_loop", "rows")])
def test_batch_matches_single_lattices(gpu, method, form):
    steps = 300
    b = BatchSimulator(DOMAINS)
    b.configure(method=method, **FORMS[form])
    assert b.config["linear"] == FORMS[form]["linear"]
    b.step(steps - 100)
    b.step(100)
    b.status()
    for i, d in enumerate(DOMAINS):
        s = _single(d, steps)
        assert np.array_equal(b.info(i), s.info())
        fb, fs = b.read_populations(i), s.read_populations()
        fluid = ~np.isin(s.info()["material"], (2, 4))
        assert np.max(np.abs(fb - fs)[:, fluid]) <= 2e-6, (i, d)
        for x, y in zip(b.read_macro(i), s.read_macro()):
            assert np.max(np.abs(x - y)[fluid]) <= 2e-6
        mb, ms = b.conservation(i)[0], s.conservation()[0]
        assert abs(mb - ms) / ms < 1e-9


def test_batch_methods_agree_on_generated_list(gpu):
    doms = generate_domains(24, 7)
    out = []
    for method in ("persistent", "domain_loop"):
        b = BatchSimulator(doms)
        b.configure(method=method)
        b.step(50)
        b.status()
        out.append([b.read_macro(i)[1] for i in range(len(doms))])
    for a, c in zip(*out):
        assert np.max(np.abs(a - c)) <= 1e-6


def test_barrier_timeout_is_reported_and_context_survives(gpu):
    b = BatchSimulator(DOMAINS)
    rc = b.inject_missing_arrival(nsteps=4, block=1, step=1, timeout_ns=200_000_000)
    assert rc == nat.LBM_ERR_TIMEOUT
    # the context is still usable: a fresh batch and a single lattice both step normally
    b2 = BatchSimulator(DOMAINS)
    b2.step(10)
    b2.status()
    s = FluidSimulator(64, 64, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)
    s.step(10)
    assert s.nonfinite_count() == 0


def test_autotune_returns_a_working_config(gpu):
    b = BatchSimulator(generate_domains(16, 3))
    cfg = b.tune(trial_steps=5)
    assert cfg["ms_per_step"] > 0 and cfg["method"] == "persistent"
    assert cfg["tile_threads_x"] % 32 == 0
    b.step(20)
    b.status()
    cfg2 = b.tune(trial_steps=5)  # cached
    assert cfg2 == cfg


def test_linear_tiles_reject_vector_cells(gpu):
    b = BatchSimulator(DOMAINS)
    with pytest.raises(nat.LbmError):
        b.configure(linear=True, cells_per_thread=4)
