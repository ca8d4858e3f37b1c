"""The C ABI from outside Python: a C99 client (tests/abi_client.c) built against include/lbm.h
and liblbm.so alone, and handles driven from several host threads at once (the ABI's threading
contract: one handle per thread, each on its own stream)."""
import os
import subprocess
import threading

import numpy as np
import pytest

from conftest import ROOT
from simuverse_gb300 import FluidSimulator

pytestmark = pytest.mark.gpu


def build_client(out_dir):
    """Compile and link tests/abi_client.c with gcc against the in-tree library."""
    from simuverse_gb300 import build

    lib = build.build()
    exe = os.path.join(str(out_dir), "abi_client")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O2",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "abi_client.c"),
                    "-L", os.path.dirname(lib), "-llbm", "-lm", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def test_c_client_drives_the_library(gpu, tmp_path):
    exe = build_client(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"


def test_handles_on_concurrent_host_threads(gpu):
    """Four threads each create, step and read their own lattice at the same time; every result
    equals the same lattice run alone (ctypes releases the interpreter lock during the calls)."""
    cfgs = [dict(mode="physics", scene="channel", tau=0.57, inlet_speed=0.05, seed=s, disk_radius=(4.0, 9.0))
            for s in range(3)] + [dict(mode="reference", scene="poiseuille", tau=0.56)]
    nx, ny = 320, 200

    def run(cfg):
        s = FluidSimulator(nx, ny, **cfg)
        s.step(150)
        out = s.read_macro()
        s.close()
        return out

    alone = [run(c) for c in cfgs]
    got = [None] * len(cfgs)
    errors = []

    def worker(i):
        try:
            got[i] = run(cfgs[i])
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(cfgs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for a, b in zip(alone, got):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
