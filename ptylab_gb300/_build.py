"""Build libptyg.so (the sm_103a kernels and the C ABI) in-tree with nvcc.

``python -m ptylab_gb300._build`` or ``build()``: each ``csrc/*.cu`` is compiled
to an object in parallel, then linked into ``ptylab_gb300/libptyg.so``.  Only
sources newer than their object are recompiled.
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
ROOT = PKG.parent
BUILD = PKG / "_build"
LIB = PKG / "libptyg.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
    # approximate division and square root (a few ulp): the intensity
    # projection and update weights stay far inside the 1e-4 parity budget
    "-prec-div=false",
    "-prec-sqrt=false",
    f"-I{ROOT / 'include'}",
    f"-I{CSRC}",
]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found; set CUDA_HOME")


def _compile(src: Path, obj: Path, extra: list[str]) -> str:
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}\n{r.stdout}")
    return r.stderr


def build(verbose: bool = False, extra_flags: list[str] | None = None, force: bool = False) -> Path:
    extra = list(extra_flags or [])
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    newest_header = max((h.stat().st_mtime for h in headers), default=0.0)
    sources = sorted(CSRC.glob("*.cu"))
    jobs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_header)
        jobs.append((src, obj, stale))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = {ex.submit(_compile, s, o, extra): s for s, o, stale in jobs if stale}
        for f in cf.as_completed(futs):
            msg = f.result()
            if verbose and msg:
                print(f"[{futs[f].name}]\n{msg}", file=sys.stderr)
    objs = [str(o) for _, o, _ in jobs]
    relink = force or not LIB.exists() or any(Path(o).stat().st_mtime > LIB.stat().st_mtime for o in objs)
    if relink:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    flags = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(verbose=v or bool(flags), extra_flags=flags, force=bool(flags)))
