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


def _close(got, expect):
    scale = abs(expect[0])
    for g, e in zip(got, expect):
        assert abs(g - e) <= REL_TOL * scale, (got, expect)


@pytest.mark.parametrize("mode", ["reference", "physics"])
def test_noalloc_sums_match_handle_sums(gpu, mode):
    import torch

    lib = nat.load()
    nx, ny = 256, 192
    sim = FluidSimulator(nx, ny, mode=mode, scene="cavity", tau=0.6, lid_speed=0.1)
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4).reshape(9, 1, 1)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # two calls in a row, on a changing state
        sim.step(40)
        expect = sim.conservation()
        if mode == "reference":
            host = sim.read_populations(np.float32)  # stored as absolute FP32 populations
        else:
            host = (sim.read_populations(np.float64) - w).astype(np.float32)  # stored as f - w
        pops = torch.from_numpy(np.ascontiguousarray(host)).cuda()
        info = torch.from_numpy(np.ascontiguousarray(sim.info()).view(np.uint8)).cuda()
        code = nat.MODES[mode]
        _noalloc(lib, pops, nat.DTYPES["f32"], code, info, nx, ny, out, stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy().tolist()
        _close(got, expect)


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
