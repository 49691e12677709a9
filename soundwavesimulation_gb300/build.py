"""In-tree build of the engine library ``libfdtd_gb300.so`` with nvcc for sm_103a.

Every translation unit compiles in parallel into ``_build/`` and links into the
package folder, where ``_lib.py`` loads it. No CMake; the only tool is nvcc.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = ("csrc/fdtd_kernels.cu", "csrc/fdtd_tb.cu", "csrc/fdtd_tb_adj.cu", "csrc/fdtd_tb_pml.cu",
           "csrc/fdtd_tb_pml_adj.cu", "csrc/fdtd_plan.cpp", "csrc/fdtd_noalloc.cu", "csrc/fdtd_optim.cu",
           "csrc/fdtd_autotune.cpp")
HEADERS = ("csrc/fdtd_device.cuh", "csrc/fdtd_internal.h", "csrc/fdtd_tb.cuh")
LIB = HERE / "libfdtd_gb300.so"
BUILD = HERE / "_build"
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")


def cuda_home() -> Path:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home:
        return Path(home)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _inputs():
    root = HERE.parent
    return [HERE / s for s in SOURCES] + [HERE / h for h in HEADERS] + [root / "include" / "fdtd_gb300.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _inputs())


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(map(str, cmd))}\n"
                           f"{res.stdout}\n{res.stderr}")
    return res.stdout + res.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library if any source is newer than it; returns its path."""
    if not force and up_to_date():
        return LIB
    nvcc = str(cuda_home() / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", *ARCH,
             "-I", str(HERE.parent / "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]
    jobs = []
    for src in SOURCES:
        path = HERE / src
        obj = BUILD / (path.stem + ".o")
        lang = ["-x", "cu"] if path.suffix == ".cpp" else []
        jobs.append((obj, [nvcc, "-c", *lang, *flags, str(path), "-o", str(obj)]))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as pool:
        logs = list(pool.map(lambda j: _run(j[1]), jobs))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, "-shared", *ARCH, *[str(o) for o, _ in jobs], "-o", str(tmp), "-cudart", "shared",
          "-Xlinker", f"-rpath,{cuda_home() / 'lib64'}"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
