"""Builds libgg.so (the sm_103a engine + its C ABI) and the oracle library.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host C++ units with g++.  Units
compile in parallel and are rebuilt when the unit or any header is newer than
its object.  Objects go to easy_graphit_gb300/_build/, the library to
easy_graphit_gb300/libgg.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgg.so"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libgg.so")
    return cand


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_lib(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    cu_flags = [*ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-fopenmp", f"-I{INCLUDE}", f"-I{CSRC}"]
    cxx_flags = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-Wall", f"-I{INCLUDE}", f"-I{CSRC}"]
    units = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    objs, cmds = [], []
    for src in units:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if not _stale(src, obj, deps):
            continue
        if src.suffix == ".cu":
            cmds.append([nvcc, *cu_flags, "-c", str(src), "-o", str(obj)])
        else:
            cmds.append(["g++", *cxx_flags, "-c", str(src), "-o", str(obj)])
    if cmds:
        workers = jobs or max(1, min(len(cmds), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            for fut in [ex.submit(_run, c) for c in cmds]:
                fut.result()
            if verbose:
                print(f"compiled {len(cmds)} unit(s)", file=sys.stderr)
    if cmds or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp", "-cudart", "static"])
        os.replace(tmp, LIB)
    return LIB


def build_cli() -> Path:
    """Builds easy_graphit_gb300/gg_app, the apps' trial-loop driver (links libgg.so)."""
    src = PKG / "cli" / "gg_app.cpp"
    exe = PKG / "gg_app"
    if not exe.exists() or any(p.stat().st_mtime > exe.stat().st_mtime for p in [src, LIB, *INCLUDE.glob("*.h")]):
        _run(["g++", "-std=c++17", "-O2", "-Wall", f"-I{INCLUDE}", str(src), "-o", str(exe),
              f"-L{PKG}", "-lgg", "-Wl,-rpath,$ORIGIN"])
    return exe


def build_oracle() -> Path:
    """Compiles the oracle's CPU restatement (test infrastructure)."""
    _run(["make", "-s", "-C", str(ORACLE), "all"])
    return ORACLE / "liboracle.so"


def build_ref_oracle() -> Path | None:
    """Compiles the reference's GAPBS code and its five apps (against the
    oracle's host-execution stand-in for BuildIt) into oracle/_ref when
    GG_REF_DIR names a reference tree (machines that only run the tests have
    none)."""
    ref_dir = os.environ.get("GG_REF_DIR")
    if not ref_dir or not (Path(ref_dir) / "runtime" / "infra_gapbs").is_dir():
        return None
    _run(["make", "-s", "-C", str(ORACLE), "ref", f"REF_DIR={ref_dir}"])
    if (Path(ref_dir) / "apps").is_dir():
        _run(["make", "-s", "-C", str(ORACLE), "apps", f"REF_DIR={ref_dir}"])
    return ORACLE / "_ref" / "ref_gapbs"


if __name__ == "__main__":
    print(build_lib(verbose=True))
    print(build_cli())
    print(build_oracle())
    print(build_ref_oracle())
