"""Build the in-tree CUDA library ``lib/libbssn_gb300.so`` for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into one shared
library with a plain C ABI (declared in ``include/bssn_gb300.h``).  No torch
headers are involved: PyTorch only supplies device memory and streams.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
LIBDIR = PACKAGE / "lib"
LIBRARY = LIBDIR / "libbssn_gb300.so"
BUILD = ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC"]


def nvcc_path() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if candidate.exists():
        return str(candidate)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jax_bssn_gb300")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    nvcc = nvcc_path()
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))
    objects = []
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *FLAGS, *ARCH, "-c", str(src), "-o", str(obj)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)

    def run(cmd):
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)
        return proc.stdout + proc.stderr

    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with concurrent.futures.ThreadPoolExecutor(workers) as pool:
            for out in pool.map(run, jobs):
                if verbose and out:
                    print(out)
    if force or jobs or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_suffix(".so.tmp")
        run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"])
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
