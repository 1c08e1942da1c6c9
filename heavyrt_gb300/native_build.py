"""Build recipe for the engine's native libraries (no cmake, no torch).

Outputs (git-ignored, rebuilt on every machine that runs them):
  heavyrt_gb300/_build/libhrt.so           CUDA engine + C ABI (include/hrt.h), sm_103a
  heavyrt_gb300/_build/libhrt_workload.so  seeded scene / ray generators
  oracle/_build/liboracle.so               CPU restatement of the reference (test oracle)
  oracle/_ref/ref_harness{,_fast}          the reference's own CPU code (only where its
  oracle/_ref/{raygen,render}_harness      sources are present)

Translation units compile in parallel; a target is rebuilt only when one of its
sources is newer than it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"
INCLUDE = ROOT / "include"

CUDA_SOURCES = ["radix_sort.cu", "build.cu", "build_batch.cu", "bvh4.cu", "trace.cu", "trace_l0.cu", "trace_l1.cu",
                "trace_l2.cu", "trace_l3.cu", "trace_w0.cu", "trace_w1.cu", "trace_w2.cu", "trace_w3.cu", "hrt_api.cu",
                "server.cu", "raygen.cu", "render.cu", "formats.cu"]
CUDA_HEADERS = ["hrt_common.cuh", "build_common.cuh", "hrt_kernels.cuh", "hrt_internal.cuh", "trace_impl.cuh",
                "raygen_common.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
HOST_CFLAGS = ["-O3", "-fPIC", "-ffp-contract=off", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build_engine(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "libhrt.so"
    headers = [CSRC / h for h in CUDA_HEADERS] + [INCLUDE / "hrt.h"]
    nvcc = _nvcc()
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(lib, objs):
        tmp = lib.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, lib)
    return lib


def build_workload(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "libhrt_workload.so"
    src = CSRC / "workload.c"
    if force or _stale(lib, [src]):
        _run(["gcc", "-std=c11", *HOST_CFLAGS, "-shared", "-o", str(lib), str(src), "-lm"])
    return lib


def build_oracle(force: bool = False) -> Path:
    out = ORACLE / "_build"
    out.mkdir(exist_ok=True)
    lib = out / "liboracle.so"
    src = ORACLE / "hrt_oracle.c"
    if force or _stale(lib, [src]):
        _run(["gcc", "-std=c11", *HOST_CFLAGS, "-fopenmp", "-shared", "-o", str(lib), str(src), "-lm"])
    return lib


def reference_root() -> Path | None:
    ref = Path(os.environ.get("HRT_REFERENCE", "/root/reference"))
    return ref if (ref / "core" / "builders" / "lbvh.cpp").exists() else None


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference's own CPU path as a checker, where its sources exist."""
    ref = reference_root()
    if ref is None:
        return None
    cmd = ["make", "-s", "-j2", "-f", "Makefile.ref", f"REF={ref}"]
    if force:
        cmd.insert(1, "-B")
    _run(cmd, cwd=ORACLE)
    return ORACLE / "_ref"


def build_all(force: bool = False) -> dict:
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        fe = ex.submit(build_engine, force)
        fw = ex.submit(build_workload, force)
        fo = ex.submit(build_oracle, force)
        fr = ex.submit(build_reference, force)
        return {"engine": fe.result(), "workload": fw.result(), "oracle": fo.result(), "reference": fr.result()}


if __name__ == "__main__":
    print(build_all())
