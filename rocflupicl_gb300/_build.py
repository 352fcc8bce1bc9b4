"""In-tree build of the native libraries (no setuptools, no cmake).

  librfmesh.so  host mesh builder (g++, OpenMP, -ffp-contract=off)
  librfgpu.so   residual engine for sm_103a (nvcc); the FP64 translation unit
                is compiled with --fmad=false so its arithmetic rounds exactly
                like the unfused reference expressions, the mixed-precision
                unit keeps FMA contraction.

Objects are rebuilt only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "_lib"

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
HOST_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA engine cannot be built")
    return cand


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return list(INCLUDE.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError("native build failed:\n" + msg)


def build_mesh(force: bool = False) -> Path:
    LIBDIR.mkdir(exist_ok=True)
    lib = LIBDIR / "librfmesh.so"
    src = CSRC / "rfmesh.cpp"
    if force or _stale(lib, [src] + _headers()):
        _run_all([["g++", *HOST_FLAGS, "-fopenmp", "-shared", f"-I{INCLUDE}", str(src),
                   "-o", str(lib)]])
    return lib


GPU_UNITS = [
    # (source, extra nvcc flags)
    ("rfgpu_host.cu", ["-Xcompiler", "-fopenmp"]),  # registration loops on host threads
    ("rfgpu_fp64.cu", ["--fmad=false"]),
    ("rfgpu_mixed.cu", []),
    ("rfgpu_meshbuild.cu", ["--fmad=false"]),
]


def build_gpu(force: bool = False) -> Path:
    LIBDIR.mkdir(exist_ok=True)
    lib = LIBDIR / "librfgpu.so"
    srcs = [CSRC / s for s, _ in GPU_UNITS]
    if not (force or _stale(lib, srcs + _headers())):
        return lib
    nvcc = _nvcc()
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    cmds, objs = [], []
    for (s, extra) in GPU_UNITS:
        obj = objdir / (Path(s).stem + ".o")
        objs.append(obj)
        cmds.append([nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                     f"-I{INCLUDE}", f"-I{CSRC}", *extra, "-c", str(CSRC / s), "-o", str(obj)])
    _run_all(cmds)
    _run_all([[nvcc, GENCODE, "-shared", *map(str, objs), "-o", str(lib), "-lcudart", "-lgomp"]])
    return lib


def build_all(force: bool = False) -> None:
    build_mesh(force)
    build_gpu(force)


if __name__ == "__main__":
    build_all(force=bool(os.environ.get("RFGPU_FORCE_BUILD")))
