"""The lattice memory pool (lbm_memory_*): lbm_destroy returns a lattice's buffers to the
library's stream-ordered pool, the next lattice of a similar size is served from it without
growing the pool, the retain limit and lbm_memory_trim give memory back, and a lattice on
recycled memory (holding a previous lattice's populations) computes what the oracle does."""
import gc

import numpy as np
import pytest

import oracle
from conftest import rel_l2
from simuverse_gb300 import FluidSimulator
from simuverse_gb300.fluid import memory_set_retain, memory_stats, memory_trim

pytestmark = pytest.mark.gpu

CHANNEL = dict(mode="physics", scene="channel", tau=0.56, inlet_speed=0.05, solid_fraction=0.05,
               disk_radius=(8.0, 32.0), seed=1234)


def _lattice_bytes(nx, ny):
    # two FP32 population buffers, flags, info records, macro planes (the small buffers aside)
    n = nx * ny
    return 2 * 9 * 4 * n + 2 * n + 16 * n + 3 * 4 * n


def test_destroyed_lattice_memory_is_reused(gpu):
    gc.collect()  # lattices of earlier tests that are no longer referenced
    nx, ny = 1024, 768
    size = _lattice_bytes(nx, ny)
    memory_set_retain(16 << 30)
    base = memory_stats()
    s = FluidSimulator(nx, ny, **CHANNEL)
    assert memory_stats()["used"] >= base["used"] + size
    s.step(10)
    s.close()
    after = memory_stats()
    assert after["used"] < base["used"] + size // 100  # returned to the pool
    assert after["reserved"] >= after["used"] + size  # and kept for the next lattice
    s2 = FluidSimulator(nx, ny, **CHANNEL)
    again = memory_stats()
    assert again["reserved"] <= after["reserved"] + (32 << 20)  # served without a new allocation
    assert again["used"] >= base["used"] + size
    s2.close()
    memory_trim()
    st = memory_stats()
    assert st["reserved"] - st["used"] < size // 2  # the lattices' memory went back


def test_retain_zero_gives_memory_back(gpu):
    gc.collect()
    size = _lattice_bytes(1024, 512)
    try:
        memory_set_retain(0)
        s = FluidSimulator(1024, 512, **CHANNEL)
        s.close()
        st = memory_stats()
        assert st["reserved"] - st["used"] < size // 2
    finally:
        memory_set_retain(16 << 30)


def test_recycled_memory_computes_as_fresh(gpu):
    """A lattice placed on the memory of a previous, differently initialised lattice of the
    same size (a moving-lid cavity that ran 300 steps) matches the oracle after 1 and 100
    steps: every buffer a step or read-back uses is initialised by lbm_create."""
    nx, ny = 384, 160
    memory_set_retain(16 << 30)
    prev = FluidSimulator(nx, ny, mode="physics", scene="cavity", tau=0.6, lid_speed=0.1)
    prev.step(300)
    prev.close()
    reserved = memory_stats()["reserved"]
    s = FluidSimulator(nx, ny, **CHANNEL)
    assert memory_stats()["reserved"] <= reserved + (32 << 20)  # the cavity's memory, reused
    info, _ = oracle.mask_physics_channel(nx, ny, 0.05, 1234, 0.05, 8.0, 32.0)
    assert np.array_equal(s.info(), info)
    ref = oracle.PhysOracle(info, 0.56, np.float32)
    assert s.conservation()[0] == pytest.approx(ref.conservation()[0], rel=1e-12)
    s.step(1)
    ref.step(1)
    rho, ux, uy = s.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert float(np.max(np.abs(rho - r_rho))) <= 1e-5
    assert float(max(np.max(np.abs(ux - r_ux)), np.max(np.abs(uy - r_uy)))) / 0.05 <= 1e-5
    s.step(99)
    ref.step(99)
    rho, ux, uy = s.read_macro()
    r_rho, r_ux, r_uy = ref.macro()
    assert rel_l2(rho, r_rho) <= 1e-4
    assert rel_l2(np.stack([ux, uy]), np.stack([r_ux, r_uy])) <= 1e-4
    s.close()
