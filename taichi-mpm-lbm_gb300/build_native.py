"""Build the sm_103a CUDA library ``fsi/_lib/libfsi_gb300.so`` in-tree.

Each translation unit in ``csrc/`` is compiled by nvcc in parallel and linked
into one shared library exporting the C ABI declared in ``include/fsi_gb300.h``.
The CUDA runtime is linked statically, so the library needs only the driver.

``-fmad=false`` keeps every float multiply and add separately rounded: the
kernels reproduce the reference's float32 operation order and must not be
contracted into fused multiply-adds.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
LIB_DIR = PKG / "fsi" / "_lib"
OBJ_DIR = LIB_DIR / "obj"
LIB = LIB_DIR / "libfsi_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["capi.cu", "lbm.cu", "mpm.cu", "mpm_sorted.cu", "coupling.cu", "context.cu", "batch.cu", "batch_step_f32.cu",
           "batch_step_f16.cu", "batch_step_bf16.cu", "batch_persist_f32.cu", "batch_persist_f16.cu",
           "batch_persist_bf16.cu", "closure.cu"]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found; set CUDA_HOME")


def _flags(verbose_ptxas: bool) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-fmad=false",
                "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _inputs() -> list[Path]:
    return [CSRC / s for s in SOURCES if (CSRC / s).exists()]


def _headers() -> list[Path]:
    return list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_headers(), Path(__file__)])


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    srcs = _inputs()
    objs = [OBJ_DIR / (s.stem + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, s)]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc(), *_flags(verbose), "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        return src.name, res.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or len(todo)) as ex:
            for name, log in ex.map(compile_one, todo):
                if verbose and log:
                    print(f"--- {name}\n{log}")
    if force or todo or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
