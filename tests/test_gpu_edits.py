"""Batched interactive edits on the GPU (lbm_apply_edits) against the same sequence of
single calls (lbm_on_click / lbm_add_obstacle / lbm_touch_* / lbm_add_external_force) and
against the oracle's restatement of d2q9_node.rs:215-300: device mask, host copy (seen
through a later row upload), and the populations after stepping."""
import numpy as np
import pytest

import oracle
from simuverse_gb300 import FluidSimulator

pytestmark = pytest.mark.gpu


def _events(rng, nx, ny, ps, n):
    ev = []
    for _ in range(n):
        r = rng.random()
        if r < 0.25:
            ev.append(("click", float(rng.uniform(-20, nx * ps + 20)), float(rng.uniform(-20, ny * ps + 20))))
        elif r < 0.35:
            ev.append(("obstacle", int(rng.integers(0, nx)), int(rng.integers(28, ny - 28))))
        elif r < 0.45:
            ev.append(("touch_begin",))
        elif r < 0.9:
            ev.append(("touch_move", float(rng.uniform(0, nx * ps)), float(rng.uniform(0, ny * ps))))
        else:
            ev.append(("force", float(rng.uniform(0, nx * ps)), float(rng.uniform(0, ny * ps)),
                       float(rng.uniform(0, nx * ps)), float(rng.uniform(0, ny * ps))))
    return ev


def _single(sim, e):
    k = e[0]
    if k == "click":
        sim.on_click(e[1:])
    elif k == "obstacle":
        sim.add_obstacle(*e[1:])
    elif k == "touch_begin":
        sim.touch_begin()
    elif k == "touch_move":
        sim.touch_move(e[1:])
    else:
        sim.add_external_force(e[1:3], e[3:5])


def _oracle(o, e):
    k = e[0]
    if k == "click":
        o.on_click(np.float32(e[1]), np.float32(e[2]))
    elif k == "obstacle":
        assert o.add_obstacle(*e[1:]) == 0
    elif k == "touch_begin":
        o.touch_begin()
    elif k == "touch_move":
        o.touch_move(e[1:])
    else:
        o.add_external_force(e[1:3], e[3:5])


@pytest.mark.parametrize("mode", ["reference", "physics"])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_batched_edits_match_single_calls(gpu, mode, seed):
    nx, ny, ps = 300, 160, 2
    kw = dict(mode=mode, scene="poiseuille" if mode == "reference" else "cavity", tau=0.6)
    a, b = FluidSimulator(nx, ny, **kw), FluidSimulator(nx, ny, **kw)
    rng = np.random.default_rng(seed)
    for batch in range(3):
        ev = _events(rng, nx, ny, ps, 40)
        for e in ev:
            _single(a, e)
        b.apply_edits(ev)
        assert np.array_equal(a.info(), b.info()), batch
        # the host copy: a single obstacle uploads whole rows from it
        x, y = int(rng.integers(0, nx)), int(rng.integers(28, ny - 28))
        a.add_obstacle(x, y)
        b.add_obstacle(x, y)
        assert np.array_equal(a.info(), b.info()), batch
        a.step(5)
        b.step(5)
    assert np.array_equal(a.read_populations(), b.read_populations())
    a.close()
    b.close()


def test_batched_edits_match_oracle(gpu):
    nx, ny, ps = 300, 160, 2
    sim = FluidSimulator(nx, ny, mode="reference", scene="poiseuille", tau=0.56)
    o = oracle.RefOracle(nx, ny, "poiseuille", tau=0.56)
    rng = np.random.default_rng(7)
    ev = _events(rng, nx, ny, ps, 120)
    n = sim.apply_edits(ev)
    for e in ev:
        _oracle(o, e)
    got = sim.info()
    assert np.array_equal(got, o.info.reshape(ny, nx))
    assert n > 0
    assert np.count_nonzero(got["material"] == 6) > 0 and np.count_nonzero(got["material"] == 4) > 0
    sim.close()


def test_bad_edit_applies_nothing(gpu):
    sim = FluidSimulator(200, 120, mode="reference", scene="poiseuille")
    before = sim.info()
    with pytest.raises(Exception):
        sim.apply_edits([("click", 150.0, 120.0), ("obstacle", 10, 5)])  # rows -23.. outside
    assert np.array_equal(sim.info(), before)
    sim.close()
