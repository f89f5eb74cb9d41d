"""Build libexoblas_gb300.so in-tree with nvcc for sm_103a.

Each translation unit under csrc/ is compiled in parallel (one -gencode,
sm_103a only) and linked into exoblas_gb300/libexoblas_gb300.so with the
CUDA runtime linked statically.  Objects go to exoblas_gb300/_build/.
An object is rebuilt when its .cu or any header under csrc/ or include/ is
newer than it.
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
OUT = PKG / "_build"
LIB = PKG / "libexoblas_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-fvisibility=hidden",
    "-I" + str(ROOT / "include"),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libexoblas_gb300")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183, "arm64": 183}


def foreign_binary(path: Path) -> bool:
    """True when `path` is an ELF object built for another CPU architecture
    (e.g. copied from an x86-64 build host to an aarch64 GPU host)."""
    import platform

    try:
        head = path.read_bytes()[:20]
    except OSError:
        return True
    if head[:4] != b"\x7fELF":
        return True
    want = _ELF_MACHINE.get(platform.machine())
    return want is not None and int.from_bytes(head[18:20], "little") != want


def _stale(obj: Path, src: Path, headers: list[Path]) -> bool:
    if not obj.exists() or foreign_binary(obj):
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in headers)


def _compile(src: Path, extra: list[str]) -> Path:
    obj = OUT / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra_flags: list[str] | None = None, jobs: int | None = None) -> Path:
    """Compile every csrc/*.cu and link libexoblas_gb300.so; returns its path."""
    OUT.mkdir(exist_ok=True)
    extra = list(extra_flags or [])
    if os.environ.get("EXOBLAS_PTXAS_VERBOSE"):
        extra += ["-Xptxas", "-v"]
    headers = _headers()
    sources = sorted(CSRC.glob("*.cu"))
    todo = [s for s in sources if extra or _stale(OUT / (s.stem + ".o"), s, headers)]
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = {ex.submit(_compile, s, extra): s for s in todo}
            for f in cf.as_completed(futs):
                f.result()
                if verbose:
                    print("compiled", futs[f].name, file=sys.stderr)
    objs = [OUT / (s.stem + ".o") for s in sources]
    if todo or not LIB.exists() or foreign_binary(LIB) or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
