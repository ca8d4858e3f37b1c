"""lbm_conservation_noalloc: the FP64 mass / momentum sums for callers that cannot
allocate device memory (their own runtime owns the device buffers, another allocator
holds the memory, or cudaMalloc's synchronisation is not affordable).  The caller passes
its device buffers; the library uses only its fixed static scratch.  Checked through the
C ABI against lbm_conservation on the same state, on two calls in a row.

This file is collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from simuverse_gb300 import FluidSimulator
from simuverse_gb300 import _native as nat

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10  # the mass tolerance of the conservation tests


def _noalloc(lib, pops, dtype, mode, info, nx, ny, out, stream):
    rc = lib.lbm_conservation_noalloc(ctypes.c_void_p(pops.data_ptr()), dtype, mode,
                                      ctypes.c_void_p(info.data_ptr()), nx, ny, ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(stream or None))
    assert rc == nat.LBM_OK, lib.lbm_last_error()


@pytest.mark.parametrize("mode,dtype", [("reference", "f32"), ("physics", "f32"), ("physics", "f64"),
                                        ("physics", "f16"), ("physics", "bf16")])
def test_noalloc_sums_match_handle_sums(gpu, mode, dtype):
    """The sums over the handle's own state buffer (its storage format: absolute FP32 in
    reference mode; f - w in FP32 / FP64 / BF16 and (f - w) * 2^10 in FP16 in physics mode)
    equal lbm_conservation's bit for bit, on two calls in a row on a changing state."""
    import torch

    lib = nat.load()
    nx, ny = 256, 192
    kw = dict(kernel="cell") if dtype in ("f16", "bf16") else {}  # the SoA layout the entry point reads
    sim = FluidSimulator(nx, ny, mode=mode, dtype=dtype, scene="cavity", tau=0.6, lid_speed=0.1, **kw)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    info = torch.from_numpy(np.ascontiguousarray(sim.info()).view(np.uint8)).cuda()
    for _ in range(2):  # two calls in a row, on a changing state
        sim.step(40)
        expect = sim.conservation()  # synchronises the handle's stream
        ptr, tiled = sim.device_populations()
        assert not tiled
        rc = lib.lbm_conservation_noalloc(ctypes.c_void_p(ptr), nat.DTYPES[dtype], nat.MODES[mode],
                                          ctypes.c_void_p(info.data_ptr()), nx, ny, ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(stream or None))
        assert rc == nat.LBM_OK, lib.lbm_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy().tolist()
        assert got == list(expect), (got, expect)


def test_noalloc_on_a_caller_buffer(gpu):
    """A population buffer the caller allocated and filled itself (absolute FP32, reference
    mode): the sums equal lbm_conservation's to within 1e-10 relative."""
    import torch

    lib = nat.load()
    nx, ny = 200, 150
    sim = FluidSimulator(nx, ny, mode="reference", scene="cavity", tau=0.6, lid_speed=0.1)
    sim.step(25)
    expect = sim.conservation()
    pops = torch.from_numpy(np.ascontiguousarray(sim.read_populations(np.float32))).cuda()
    info = torch.from_numpy(np.ascontiguousarray(sim.info()).view(np.uint8)).cuda()
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    _noalloc(lib, pops, nat.DTYPES["f32"], nat.MODES["reference"], info, nx, ny, out,
             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy().tolist()
    for g, e in zip(got, expect):
        assert abs(g - e) <= REL_TOL * abs(expect[0]), (got, expect)


def test_noalloc_rejects_oversized_and_bad_arguments(gpu):
    import torch

    lib = nat.load()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    o = ctypes.c_void_p(out.data_ptr())
    assert lib.lbm_conservation_noalloc(p, 0, 0, None, 65536, 32769, o, None) == nat.LBM_ERR_ARG  # > 2^30 cells
    assert b"2^30" in lib.lbm_last_error()
    assert lib.lbm_conservation_noalloc(p, 0, 1, None, 4, 4, o, None) == nat.LBM_ERR_ARG  # physics needs info
    assert lib.lbm_conservation_noalloc(None, 0, 0, None, 4, 4, o, None) == nat.LBM_ERR_ARG
    assert lib.lbm_conservation_noalloc(p, 2, 0, None, 4, 4, o, None) == nat.LBM_ERR_ARG  # reference mode is FP32
