"""The C ABI without a GPU: the library loads, exports every declared symbol, validates
arguments without aborting, and its host-side mask logic (masks, obstacle discs, force
strokes) agrees with the oracle's restatement of lattice.rs / d2q9_node.rs."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from conftest import ROOT


def _declared(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(native):
    names = _declared("lbm.h")
    assert len(names) > 30
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_abi_version_and_defaults(native):
    from simuverse_gb300 import _native as nat

    assert native.lbm_abi_version() == 1
    p = nat.LbmParams()
    native.lbm_params_default(ctypes.byref(p))
    assert (p.nx, p.ny) == (600, 375)  # 1200x750 canvas, lattice_pixel_size 2
    assert p.tau == pytest.approx(0.56)
    assert p.lid_speed == pytest.approx(0.13) and p.inlet_speed == pytest.approx(0.12)


@pytest.mark.parametrize("field,value", [("nx", 2), ("ny", 70000), ("mode", 5), ("dtype", 9), ("scene", 3),
                                         ("tau", 0.0), ("pixel_size", 0)])
def test_create_rejects_bad_params(native, field, value):
    from simuverse_gb300 import _native as nat

    p = nat.LbmParams()
    native.lbm_params_default(ctypes.byref(p))
    setattr(p, field, value)
    h = ctypes.c_void_p()
    rc = native.lbm_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == nat.LBM_ERR_ARG
    assert h.value is None
    assert len(native.lbm_last_error()) > 0


@pytest.mark.parametrize("mode,dtype,kernel,rounding", [
    (0, 0, 0, 1),  # reference mode
    (1, 0, 0, 1),  # physics FP32: nothing to round
    (1, 1, 0, 1),  # physics FP64
    (1, 2, 3, 1),  # FP16 on the bulk-copy kernel
    (1, 3, 2, 1),  # BF16 on the four-cell kernel
    (1, 2, 0, 7),  # unknown rounding
])
def test_create_rejects_bad_rounding(native, mode, dtype, kernel, rounding):
    from simuverse_gb300 import _native as nat

    p = nat.LbmParams()
    native.lbm_params_default(ctypes.byref(p))
    p.nx, p.ny, p.mode, p.dtype, p.kernel, p.rounding = 128, 64, mode, dtype, kernel, rounding
    p.scene = nat.SCENES["periodic"] if mode == 1 else 0
    h = ctypes.c_void_p()
    assert native.lbm_create(ctypes.byref(p), ctypes.byref(h)) == nat.LBM_ERR_ARG
    assert h.value is None
    assert "round" in native.lbm_last_error().decode()


def test_scene_disks_are_the_channel_obstacles(native):
    """The disk list lbm_create uploads for a channel: non-overlapping with a 2-cell gap, and
    its rasterisation is exactly the obstacle set of the host mask."""
    from simuverse_gb300 import _native as nat

    p = nat.LbmParams()
    native.lbm_params_default(ctypes.byref(p))
    p.nx, p.ny, p.mode, p.scene, p.seed = 300, 120, 1, nat.SCENES["channel"], 42
    p.solid_fraction, p.disk_rmin, p.disk_rmax, p.inlet_speed = 0.06, 4.0, 12.0, 0.05
    n = ctypes.c_int32()
    assert native.lbm_scene_disks(ctypes.byref(p), None, 0, ctypes.byref(n)) == 0
    assert n.value > 5
    d = np.empty((n.value, 3), np.float64)
    assert native.lbm_scene_disks(ctypes.byref(p), nat.ptr(d), n.value, ctypes.byref(n)) == 0
    for i in range(len(d)):
        for j in range(i):
            assert np.hypot(d[i, 0] - d[j, 0], d[i, 1] - d[j, 1]) >= d[i, 2] + d[j, 2] + 2.0
    mask = np.empty((p.ny, p.nx), dtype=nat.INFO_DTYPE)
    nat.check(native.lbm_build_mask(ctypes.byref(p), nat.ptr(mask)))
    y, x = np.mgrid[0:p.ny, 0:p.nx].astype(np.float64)
    inner = (x >= 1) & (x <= p.nx - 2) & (y >= 1) & (y <= p.ny - 2)
    ras = np.zeros((p.ny, p.nx), bool)
    for cx, cy, r in d:
        ras |= inner & ((x - cx) ** 2 + (y - cy) ** 2 <= r * r)
    assert np.array_equal(ras, mask["material"] == 4)
    assert ras.sum() >= 0.06 * p.nx * p.ny


def test_header_serves_a_c99_client(native, tmp_path):
    """include/lbm.h is plain C99: the C client (tests/abi_client.c) compiles with warnings as
    errors and links against liblbm.so alone (it runs on a GPU in tests/test_gpu_abi.py)."""
    import shutil
    import subprocess

    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    from test_gpu_abi import build_client

    exe = build_client(tmp_path)
    assert os.path.exists(exe)
    out = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    used = sorted(set(re.findall(r"\b(lbm_[a-z0-9_]+)", out)))
    assert "lbm_create" in used and "lbm_read_macro" in used and "lbm_memory_stats" in used


def test_null_handles_are_errors(native):
    from simuverse_gb300 import _native as nat

    assert native.lbm_step(None, 1) == nat.LBM_ERR_ARG
    assert native.lbm_reset(None) == nat.LBM_ERR_ARG
    assert native.lbm_destroy(None) == nat.LBM_OK
    assert native.lbm_create(None, None) == nat.LBM_ERR_ARG


def _mask(native, nx, ny, mode, scene, **kw):
    from simuverse_gb300 import _native as nat

    p = nat.LbmParams()
    native.lbm_params_default(ctypes.byref(p))
    p.nx, p.ny, p.mode, p.scene = nx, ny, mode, scene
    for k, v in kw.items():
        setattr(p, k, v)
    out = np.zeros((ny, nx), nat.INFO_DTYPE)
    nat.check(native.lbm_build_mask(ctypes.byref(p), nat.ptr(out)))
    return out


@pytest.mark.parametrize("scene,nx,ny", [("poiseuille", 600, 375), ("poiseuille", 97, 61), ("cavity", 256, 256),
                                         ("custom", 17, 9)])
def test_reference_masks_match_oracle(native, scene, nx, ny):
    sc = {"poiseuille": 0, "cavity": 1, "custom": 2}[scene]
    got = _mask(native, nx, ny, 0, sc, lid_speed=0.1, inlet_speed=0.12)
    assert np.array_equal(got, oracle.mask_reference(nx, ny, scene, 0.1, 0.12))


def test_physics_masks_match_oracle(native):
    assert np.array_equal(_mask(native, 130, 70, 1, 1, lid_speed=0.1), oracle.mask_physics_cavity(130, 70, 0.1))
    for seed in (0, 1, 1234):
        got = _mask(native, 700, 300, 1, 3, inlet_speed=0.05, seed=seed, solid_fraction=0.05,
                    disk_rmin=8.0, disk_rmax=32.0)
        ref, _ = oracle.mask_physics_channel(700, 300, 0.05, seed, 0.05, 8.0, 32.0)
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("nx,ny,seed,frac,rmin,rmax", [
    (4096, 4096, 1234, 0.05, 8.0, 32.0),  # the channel workload of the benchmark
    (333, 257, 7, 0.2, 3.0, 3.0),         # equal radii, dense
    (500, 90, 99, 0.3, 0.0, 2.5),         # radii below three cells, very dense
    (257, 511, 5, 0.12, 4.25, 19.75),     # quarter-cell radii
    (40, 30, 3, 0.1, 30.0, 60.0),         # no disk fits: an empty list
])
def test_channel_masks_match_oracle(native, nx, ny, seed, frac, rmin, rmax):
    """The disk sampler (grid-pruned overlap test, row-span cell count) accepts exactly the
    disks of the oracle's plain rejection sampler, so the masks are equal record for record."""
    got = _mask(native, nx, ny, 1, 3, inlet_speed=0.05, seed=seed, solid_fraction=frac, disk_rmin=rmin,
                disk_rmax=rmax)
    ref, n = oracle.mask_physics_channel(nx, ny, 0.05, seed, frac, rmin, rmax)
    assert np.array_equal(got, ref)
    from simuverse_gb300.fluid import scene_disks

    d = scene_disks(nx, ny, mode="physics", scene="channel", inlet_speed=0.05, seed=seed, solid_fraction=frac,
                    disk_radius=(rmin, rmax))
    assert len(d) == n


def test_obstacle_disc_matches_oracle(native):
    from simuverse_gb300 import _native as nat

    nx, ny = 200, 150
    base = oracle.mask_reference(nx, ny, "cavity")
    for x, y in ((100, 70), (28, 28), (171, 121), (0, 40)):
        a = base.copy()
        nat.check(native.lbm_mask_add_obstacle(nx, ny, nat.ptr(a), x, y))
        host, dev = base.copy(), base.copy()
        assert oracle.lib().lo_add_obstacle(nx, ny, oracle._p(host), oracle._p(dev), x, y) == 0
        assert np.array_equal(a, host) and np.array_equal(a, dev)
    bad = base.copy()
    assert native.lbm_mask_add_obstacle(nx, ny, nat.ptr(bad), 100, 10) == nat.LBM_ERR_ARG


@pytest.mark.parametrize("pos,pre,ps", [((400.0, 300.0), (380.0, 290.0), 4), ((100.0, 100.0), (120.0, 60.0), 2),
                                        ((5.0, 5.0), (50.0, 40.0), 3), ((790.0, 10.0), (700.0, 50.0), 4),
                                        ((300.0, 300.0), (300.0, 300.0), 4)])
def test_force_stroke_matches_oracle(native, pos, pre, ps):
    from simuverse_gb300 import _native as nat

    nx, ny = 200, 150
    a = oracle.mask_reference(nx, ny, "poiseuille")
    b = a.copy()
    n = native.lbm_mask_force_stroke(nx, ny, ps, nat.ptr(a), pos[0], pos[1], pre[0], pre[1])
    assert n >= 0
    oracle.lib().lo_add_external_force(nx, ny, ps, oracle._p(b), pos[0], pos[1], pre[0], pre[1])
    assert np.array_equal(a, b)


def test_force_stroke_rejects_unit_pixel(native):
    from simuverse_gb300 import _native as nat

    a = oracle.mask_reference(50, 40, "cavity")
    assert native.lbm_mask_force_stroke(50, 40, 1, nat.ptr(a), 10.0, 10.0, 20.0, 20.0) == nat.LBM_ERR_ARG


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from simuverse_gb300 import _native as nat

    monkeypatch.setattr(nat, "_lib", None)
    monkeypatch.setattr(nat, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(RuntimeError):
        nat.load()


def test_python_params_and_scene_disks():
    from simuverse_gb300.fluid import make_params, scene_disks

    p = make_params(300, 120, mode="physics", dtype="f16", scene="channel", tau=0.7, inlet_speed=0.05, seed=42,
                    solid_fraction=0.06, disk_radius=(4.0, 12.0), kernel="tiled", rounding="stochastic")
    assert (p.nx, p.ny, p.mode, p.dtype, p.scene, p.kernel, p.rounding) == (300, 120, 1, 2, 3, 5, 1)
    assert p.tau == pytest.approx(0.7) and p.seed == 42
    d = scene_disks(300, 120, mode="physics", scene="channel", inlet_speed=0.05, seed=42, solid_fraction=0.06,
                    disk_radius=(4.0, 12.0))
    assert d.shape[1] == 3 and len(d) > 5
    assert np.all((d[:, 2] >= 4.0) & (d[:, 2] <= 12.0))
    assert len(scene_disks(64, 64, mode="physics", scene="cavity")) == 0
    with pytest.raises(KeyError):
        make_params(64, 64, rounding="sometimes")


def test_no_gpu_fails_loudly():
    """Without a usable GPU every entry point that needs one returns an error (no CPU fallback)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from simuverse_gb300 import BatchSimulator, FluidSimulator, generate_domains
    from simuverse_gb300 import _native as nat
    from simuverse_gb300.closure import Closure

    with pytest.raises(nat.LbmError):
        FluidSimulator(64, 64, mode="physics", scene="channel")
    with pytest.raises(nat.LbmError):
        BatchSimulator(generate_domains(4, 1))
    with pytest.raises(nat.LbmError):
        Closure(64, 64)


def test_python_tables_match_the_header():
    """The Python mirror's name tables and status codes are the header's #define values."""
    import re

    from simuverse_gb300 import _native as nat

    text = open(os.path.join(ROOT, "include", "lbm.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (LBM_[A-Z0-9_]+) +\(?(-?\d+)\)?", text)}
    for prefix, table in (("LBM_MODE_", nat.MODES), ("LBM_DTYPE_", nat.DTYPES), ("LBM_SCENE_", nat.SCENES),
                          ("LBM_KERNEL_", nat.KERNELS), ("LBM_COLLISION_", nat.COLLISIONS),
                          ("LBM_ROUNDING_", nat.ROUNDINGS), ("LBM_ARITH_", nat.ARITHS)):
        header = {k[len(prefix):].lower(): v for k, v in defs.items() if k.startswith(prefix)}
        assert header == table, prefix
    for name in ("ARG", "CUDA", "TIMEOUT", "NAN", "IO", "STATE", "NOMEM"):
        assert defs["LBM_ERR_" + name] == getattr(nat, "LBM_ERR_" + name)


@pytest.mark.parametrize("dtype,nx,kernel", [
    (0, 128, 6),   # the ring-staged tiled step on FP32
    (2, 100, 6),   # nx % 64
    (2, 100, 5),   # the tiled step, nx % 64
    (2, 128, 7),   # unknown kernel
])
def test_create_rejects_kernels_where_they_do_not_apply(native, dtype, nx, kernel):
    from simuverse_gb300 import _native as nat

    p = nat.LbmParams()
    native.lbm_params_default(ctypes.byref(p))
    p.nx, p.ny, p.mode, p.dtype, p.kernel = nx, 64, 1, dtype, kernel
    p.scene = nat.SCENES["periodic"]
    h = ctypes.c_void_p()
    assert native.lbm_create(ctypes.byref(p), ctypes.byref(h)) == nat.LBM_ERR_ARG
    assert h.value is None
    assert "kernel" in native.lbm_last_error().decode()
