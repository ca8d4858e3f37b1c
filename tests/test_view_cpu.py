"""Consumers of the macro field without a GPU: the particle grid and initial particle
layout of the library's host code against the oracle (lib.rs:248-316), FP16 rounding of
the oracle against numpy's, and the oracle's particle update against an independent
numpy restatement of particle_update.wgsl."""
import ctypes

import numpy as np
import pytest

import oracle


@pytest.mark.parametrize("cw,ch,count", [(1200, 750, 10000), (400, 240, 3000), (256, 256, 205000), (7, 5, 2)])
def test_particle_grid_matches_oracle(native, cw, ch, count):
    a, b = ctypes.c_int32(), ctypes.c_int32()
    assert native.lbm_particles_grid(cw, ch, count, ctypes.byref(a), ctypes.byref(b)) == 0
    assert (a.value, b.value) == oracle.particles_grid(cw, ch, count)
    # at least `count` particles, about the canvas aspect
    assert a.value * b.value >= count


@pytest.mark.parametrize("life", [60.0, 1.0, 0.0])
def test_particle_init_matches_oracle(native, life):
    from simuverse_gb300.view import particle_params

    p = particle_params(400, 240, count=3000, life_time=life, seed=11)
    nx, ny = oracle.particles_grid(400, 240, 3000)
    out = np.empty((nx * ny, 6), np.float32)
    assert native.lbm_particles_init_state(ctypes.byref(p), nx, ny, out.ctypes.data_as(ctypes.c_void_p)) == 0
    ref = oracle.particles_init(400, 240, nx, ny, life, 11)
    assert np.array_equal(out, ref)
    # grid column x, row y at record x * ny + y, jittered by at most one grid step
    step_x, step_y = np.float32(400) / (nx - 1), np.float32(240) / (ny - 1)
    gx = np.repeat(np.arange(nx), ny) * step_x
    gy = np.tile(np.arange(ny), nx) * step_y
    assert np.all(np.abs(out[:, 0] - gx) <= step_x * 1.0001) and np.all(np.abs(out[:, 1] - gy) <= step_y * 1.0001)
    if life > 1.0:
        assert np.array_equal(out[:, 2:4], out[:, 0:2]) and out[:, 4].min() >= 0 and out[:, 4].max() <= life
    else:
        assert np.all(out[:, 4] == 0) and np.all((out[:, 2] >= 0) & (out[:, 2] < step_x))


def test_h16_matches_numpy():
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.standard_normal(2000) * 10.0 ** rng.integers(-9, 5, 2000),
                        np.array([0.0, -0.0, 65504.0, 65519.9, 65520.0, 6.1e-5, 5.96e-8, 2.98e-8, 1e-9])]).astype(np.float32)
    L = oracle.lib()
    got = np.array([L.lo_h16(float(x)) for x in v], np.float32)
    with np.errstate(over="ignore"):
        ref = v.astype(np.float16).astype(np.float32)
    assert np.array_equal(got, ref)


def _np_update(ux, uy, lp, life_time, speed, point, cw, ch, pois, st, canvas):
    """particle_update.wgsl:55-87 in numpy float32 scalars (each operation rounds)."""
    f32 = np.float32
    ny, nx = ux.shape
    u16, v16 = ux.astype(np.float16).astype(f32), uy.astype(np.float16).astype(f32)

    def tex(a, i, j):
        return a[min(max(j, 0), ny - 1), min(max(i, 0), nx - 1)]

    for k in range(st.shape[0]):
        px, py, ix, iy, life, fade = (f32(v) for v in st[k])
        if life <= f32(0.1):
            st[k] = (ix, iy, ix, iy, f32(life_time), f32(0))
            continue
        life = f32(life - f32(1))
        if fade < f32(1):
            fade = f32(fade + f32(0.1)) if fade < f32(0.95) else f32(1)
        gx, gy = f32(f32(px / f32(lp)) - f32(0.5)), f32(f32(py / f32(lp)) - f32(0.5))
        mx, my = int(np.floor(gx)), int(np.floor(gy))
        fx, fy = f32(gx - f32(mx)), f32(gy - f32(my))
        w = [f32(f32(1 - fx) * f32(1 - fy)), f32(f32(1 - fx) * fy), f32(fx * f32(1 - fy)), f32(fx * fy)]
        taps = [(mx, my), (mx, my + 1), (mx + 1, my), (mx + 1, my + 1)]
        v = []
        for a in (u16, v16):
            s = f32(0)
            for t, (i, j) in enumerate(taps):
                s = f32(s + f32(tex(a, i, j) * w[t])) if t else f32(tex(a, i, j) * w[t])
            v.append(s)
        px, py = f32(px + f32(v[0] * f32(speed))), f32(py + f32(v[1] * f32(speed)))
        st[k] = (px, py, ix, iy, life, fade)
        sp = f32(abs(v[0]) + abs(v[1]))
        if (not pois and sp < 0) or (pois and sp < f32(0.015)):
            continue
        x0, y0 = int(px) - point // 2, int(py) - point // 2
        for dx in range(point):
            for dy in range(point):
                cx, cy = x0 + dx, y0 + dy
                if 0 <= cx < cw and 0 <= cy < ch:
                    canvas[cy, cx] = (fade, v[0], v[1])


def test_oracle_particle_update_matches_numpy_restatement():
    rng = np.random.default_rng(3)
    nx, ny, lp, cw, ch = 20, 12, 2, 40, 24
    ux = (0.08 * rng.standard_normal((ny, nx))).astype(np.float32)
    uy = (0.08 * rng.standard_normal((ny, nx))).astype(np.float32)
    st = oracle.particles_init(cw, ch, 9, 6, 5.0, 2)
    st[:, 5] = rng.random(st.shape[0]).astype(np.float32)
    a, b = st.copy(), st.copy()
    ca, cb = np.zeros((ch, cw, 3), np.float32), np.zeros((ch, cw, 3), np.float32)
    for it in range(8):
        oracle.particles_update(ux, uy, False, lp, 5.0, 4.15, 3, cw, ch, True, a, ca)
        _np_update(ux, uy, lp, 5.0, 4.15, 3, cw, ch, True, b, cb)
        assert np.array_equal(a, b), it
        assert np.array_equal(ca, cb), it
    assert np.count_nonzero(ca[..., 0]) > 0


def test_particle_host_functions_reject_bad_input(native):
    from simuverse_gb300.view import particle_params

    a, b = ctypes.c_int32(), ctypes.c_int32()
    for cw, ch, count in ((0, 10, 10), (10, 0, 10), (10, 10, 0), (-5, 10, 10)):
        assert native.lbm_particles_grid(cw, ch, count, ctypes.byref(a), ctypes.byref(b)) < 0
    p = particle_params(40, 30, count=1)
    out = np.empty((4, 6), np.float32)
    # a 1 x 1 grid has no spacing (the reference would divide by zero): refused
    assert native.lbm_particles_init_state(ctypes.byref(p), 1, 1, out.ctypes.data_as(ctypes.c_void_p)) < 0
    assert native.lbm_particles_init_state(None, 2, 2, out.ctypes.data_as(ctypes.c_void_p)) < 0
