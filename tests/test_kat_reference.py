"""Hand-computed known answers for one reference-mode collide (collide_stream.wgsl:40-87).

Each case gives the nine populations a fluid cell pulls, tau, and an optional force (an
external-force cell, material 6, of lattice.rs:15-24).  ``collide_by_hand`` evaluates the
shader's expressions in the shader's order with every intermediate rounded to float32 and
the constants written in simuverse/src/fluid/mod.rs:31-49 (truncated weights 0.444444,
0.111111, 0.0277777; maxima 0.6, 0.2222, 0.1111; omega = 1 / tau in f32).  The expected
bit patterns below were taken from that evaluation once and are asserted literally, so the
known answers do not depend on any code under test:

* ``bulk``: an ordinary fluid cell;
* ``rho_clamp``: pulled density 1.22, clamped to 1.2 (collide_stream.wgsl:49);
* ``force``: velocity replaced by F / (2 rho) and F_i = 3 w_i e_i . F added (:55-71), the
  countdown block_iter 5 -> 4;
* ``force_clamp``: as ``force`` with a force large enough that the population clamp of
  :79-83 sets population 1 to its maximum 0.2222 and populations 6 and 7 to 0.

The oracle must reproduce them bit for bit (CPU test); the exact CUDA step bit for bit and
the fast one within 1e-5 relative (GPU tests).
"""
import numpy as np
import pytest

import oracle

f32 = np.float32
W = [f32(0.444444)] + [f32(0.111111)] * 4 + [f32(0.0277777)] * 4
MAXV = [f32(0.6)] + [f32(0.2222)] * 4 + [f32(0.1111)] * 4
EX = [0, 1, 0, -1, 0, 1, -1, -1, 1]
EY = [0, 0, -1, 0, 1, -1, -1, 1, 1]

CASES = {
    "bulk": ([0.43, 0.12, 0.105, 0.1, 0.115, 0.03, 0.026, 0.0275, 0.029], 0.6, None),
    "rho_clamp": ([0.52, 0.15, 0.13, 0.11, 0.16, 0.04, 0.03, 0.035, 0.045], 0.56, None),
    "force": ([0.43, 0.21, 0.105, 0.1, 0.115, 0.03, 0.026, 0.0275, 0.029], 0.6, (0.12, -0.05)),
    "force_clamp": ([0.43, 0.21, 0.105, 0.01, 0.115, 0.03, 0.026, 0.0275, 0.029], 0.6, (0.3, 0.02)),
}

# (rho, ux, uy, populations 0..8) as IEEE float32 bit patterns
EXPECTED = {
    "bulk": (0x3F7B851F, 0x3CD49DE4, 0x3C2F18A2,
             [0x3EE1687F, 0x3DEE7BFE, 0x3DD910FF, 0x3DCFC3B2, 0x3DE34E6D, 0x3CE1CC5F, 0x3CBF7A3F, 0x3CCD5183,
              0x3D0081B3]),
    "rho_clamp": (0x3F99999A, 0x3D4CCCCE, 0x3D088889,
                  [0x3F09E4F5, 0x3E211E00, 0x3DE57708, 0x3DF05086, 0x3E0B5B72, 0x3CFC8108, 0x3CB93682, 0x3CEBECD2,
                   0x3D263C92]),
    "force": (0x3F8947AF, 0x3D652596, 0xBCBEF4A8,
              [0x3F00DED2, 0x3E08DACC, 0x3E225CFA, 0x3D770BBE, 0x3DB9EAE9, 0x3D687799, 0x3CB0DC03, 0x3BD43D68,
               0x3D27D8AB]),
    "force_clamp": (0x3F7B851E, 0x3E1C55FD, 0x3C26C21E,
                    [0x3ED4C33B, 0x3E638866, 0x3DBF518F, 0x3B9800F0, 0x3DE3BA3A, 0x3D910B48, 0x00000000, 0x00000000,
                     0x3DA187D0]),
}

NX = NY = 4
CX, CY = 1, 1  # the cell under test


def bits(v) -> int:
    return int(np.asarray(v, np.float32).view(np.uint32))


def collide_by_hand(f, tau, force=None):
    """collide_stream.wgsl:40-87 for one cell, every operation rounded to float32."""
    f = [f32(v) for v in f]
    omega = f32(1.0) / f32(tau)  # mod.rs:34
    rho, vx, vy = f32(0), f32(0), f32(0)
    for i in range(9):  # :40-46
        rho = f32(rho + f[i])
        vx = f32(vx + f32(f32(EX[i]) * f[i]))
        vy = f32(vy + f32(f32(EY[i]) * f[i]))
    rho = min(max(rho, f32(0.8)), f32(1.2))  # :49
    vx, vy = f32(vx / rho), f32(vy / rho)  # :51
    F = [f32(0)] * 9
    if force is not None:  # :55-71
        fx, fy = f32(force[0]), f32(force[1])
        vx = f32(f32(fx * f32(0.5)) / rho)
        vy = f32(f32(fy * f32(0.5)) / rho)
        F = [f32(f32(W[i] * f32(3.0)) * f32(f32(f32(EX[i]) * fx) + f32(f32(EY[i]) * fy))) for i in range(9)]
    usqr = f32(f32(1.5) * f32(f32(vx * vx) + f32(vy * vy)))  # :76
    out = []
    for i in range(9):  # :77-87 with equilibrium() of :18-22
        eu = f32(f32(f32(EX[i]) * vx) + f32(f32(EY[i]) * vy))
        feq = f32(f32(rho * W[i]) * f32(f32(f32(f32(1.0) + f32(f32(3.0) * eu)) + f32(f32(4.5) * f32(eu * eu))) - usqr))
        t = f32(f32(f[i] - f32(omega * f32(f[i] - feq))) + F[i])
        if t > MAXV[i]:
            t = MAXV[i]
        elif t < f32(0):
            t = f32(0)
        out.append(t)
    return rho, vx, vy, out


def lattice(case):
    """A 4x4 all-fluid lattice (periodic pull) whose cell (1, 1) pulls the case's populations;
    the info records and the populations as absolute FP32 planes."""
    f, tau, force = CASES[case]
    info = np.zeros((NY, NX), oracle.INFO_DTYPE)
    info["material"] = 1
    info["block_iter"] = -1
    if force is not None:
        info[CY, CX] = (6, 5, force[0], force[1])
    A = np.empty((9, NY, NX), np.float32)
    for j in range(9):
        A[j] = W[j]
        A[j, (CY - EY[j]) % NY, (CX - EX[j]) % NX] = f32(f[j])  # streaming_in source of direction j
    return info, A, tau


@pytest.mark.parametrize("case", sorted(CASES))
def test_hand_evaluation_gives_the_literals(case):
    rho, vx, vy, out = collide_by_hand(*CASES[case])
    e_rho, e_vx, e_vy, e_out = EXPECTED[case]
    assert (bits(rho), bits(vx), bits(vy)) == (e_rho, e_vx, e_vy)
    assert [bits(v) for v in out] == e_out


def test_clamps_are_exercised():
    assert bits(collide_by_hand(*CASES["rho_clamp"])[0]) == bits(f32(1.2))
    out = collide_by_hand(*CASES["force_clamp"])[3]
    assert bits(out[1]) == bits(f32(0.2222)) and out[6] == 0 and out[7] == 0


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_reproduces_known_answers(case):
    info, A, tau = lattice(case)
    ref = oracle.RefOracle(NX, NY, "custom", tau=tau, info=info)
    ref.info[...] = info  # after init.wgsl, which clears forcing cells with a countdown
    ref.bufs[ref.cur][...] = A
    ref.step(1)
    e_rho, e_vx, e_vy, e_out = EXPECTED[case]
    rho, ux, uy = ref.macro()
    assert (bits(rho[CY, CX]), bits(ux[CY, CX]), bits(uy[CY, CX])) == (e_rho, e_vx, e_vy)
    assert [bits(v) for v in ref.populations[:, CY, CX]] == e_out
    if CASES[case][2] is not None:
        assert ref.info[CY, CX]["block_iter"] == 4 and ref.info[CY, CX]["material"] == 6


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["exact", "fast"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_reproduces_known_answers(gpu, case, arith):
    from simuverse_gb300 import FluidSimulator

    info, A, tau = lattice(case)
    sim = FluidSimulator(NX, NY, mode="reference", scene="custom", tau=tau, arith=arith)
    sim.set_info(info)
    sim.write_populations(A)
    sim.step(1)
    e_rho, e_vx, e_vy, e_out = EXPECTED[case]
    rho, ux, uy = (a[CY, CX] for a in sim.read_macro())
    out = sim.read_populations()[:, CY, CX]
    if arith == "exact":
        assert (bits(rho), bits(ux), bits(uy)) == (e_rho, e_vx, e_vy)
        assert [bits(v) for v in out] == e_out
    else:
        want = np.array(e_out, np.uint32).view(np.float32)
        for got, exp in ((rho, e_rho), (ux, e_vx), (uy, e_vy)):
            exp = np.uint32(exp).view(np.float32)
            assert abs(float(got) - float(exp)) <= 1e-5 * max(abs(float(exp)), 1e-3)
        assert np.max(np.abs(out - want)) <= 1e-6
        # the clamps give the same values: maxima and zeros are exact
        clamped = (want == 0) | np.isin(want, np.array(MAXV, np.float32))
        assert np.array_equal(out[clamped], want[clamped])
    if CASES[case][2] is not None:
        got = sim.info()[CY, CX]
        assert got["block_iter"] == 4 and got["material"] == 6
    sim.close()
