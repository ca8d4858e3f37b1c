"""Build liblbm.so (the CUDA library behind include/lbm.h) in-tree with nvcc for sm_103a.

Translation units are compiled in parallel; the shared object lands in
simuverse_gb300/_lib/liblbm.so.  Host code is compiled with -ffp-contract=off so that the
mask and force-stroke geometry rounds like the Rust code it mirrors.

build(variant="bounds") builds liblbm_bounds.so, the same sources with LBM_BOUNDS_CHECK: the
step kernels check every population, flag and info index against its buffer and record the
out-of-range ones instead of accessing them (lbm_bounds_report).  A debugging build, slower;
select it with SIMUVERSE_LBM_VARIANT=bounds before the package loads the library.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "liblbm.so")
VARIANTS = {None: ("liblbm.so", "obj", []), "bounds": ("liblbm_bounds.so", "obj_bounds", ["-DLBM_BOUNDS_CHECK"])}


def lib_path(variant=None) -> str:
    return os.path.join(OUT, VARIANTS[variant][0])
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["lbm_kernels.cu", "lbm_step_vec.cu", "lbm_step_bulk.cu", "lbm_batch.cu", "lbm_noalloc.cu", "lbm_closure.cu", "lbm_view.cu", "lbm_api.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; liblbm.so cannot be built")
    return cand


def _deps():
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force: bool = False, verbose: bool = False, variant=None) -> str:
    name, obj_name, defines = VARIANTS[variant]
    lib = os.path.join(OUT, name)
    if not force and not _stale(lib):
        return lib
    nvcc = _nvcc()
    obj_dir = os.path.join(OUT, obj_name)
    os.makedirs(obj_dir, exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")] + defines
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + common + ARCH + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd += ["--expt-relaxed-constexpr"]
            if verbose:
                cmd += ["-Xptxas", "-v"]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError("nvcc failed on " + ", ".join(failed))
    tmp = lib + ".tmp.%d" % os.getpid()
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                variant="bounds" if "--bounds" in sys.argv else None))
