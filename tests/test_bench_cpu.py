"""bench.py host logic: the step kernel AUTO runs, and the DRAM traffic it reports comes only from
a committed ncu summary of the same configuration."""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _args(**kw):
    d = dict(dtype="f32", nx=4096, ny=4096, kernel="auto", rounding="nearest")
    d.update(kw)
    return argparse.Namespace(**d)


def test_effective_kernel():
    assert bench.effective_kernel(_args()) == "cell"
    assert bench.effective_kernel(_args(dtype="f64")) == "cell"
    assert bench.effective_kernel(_args(dtype="f16", nx=8192)) == "tiled"
    assert bench.effective_kernel(_args(dtype="bf16", nx=1000)) == "vec2"
    assert bench.effective_kernel(_args(kernel="vec4")) == "vec4"


def test_traffic_only_for_the_profiled_configuration():
    assert bench.committed_traffic(_args())["bytes_per_launch_scaled"] == 1200069376
    f16 = bench.committed_traffic(_args(dtype="f16", nx=8192, ny=8192, rounding="stochastic"))
    assert f16["bytes_per_launch_scaled"] > 2415919104  # above the 36 B/cell algorithmic bytes
    assert bench.committed_traffic(_args(dtype="f16")) is None  # 4096^2 FP16 was not profiled
    assert bench.committed_traffic(_args(nx=8192, ny=8192)) is None
    assert bench.committed_traffic(_args(kernel="vec4")) is None
