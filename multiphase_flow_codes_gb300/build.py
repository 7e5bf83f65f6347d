"""Build the engine's shared library, ``_lib/liblbm_gb300.so``, from ``csrc/``.

The library is plain CUDA C++ for sm_103a behind the C ABI of
``include/lbm.h``; it links the CUDA runtime statically and cuFFT (used only
by the statistics entry) dynamically.  Translation units compile in parallel.  The particle and
forcing units are built with ``-fmad=false`` so that the geometry deciding
solid flags, links and refill events rounds exactly like the CPU restatement
used by the tests.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "liblbm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", str(PKG.parent / "include")]
# (source, extra flags)
UNITS = [
    ("lbm_fluid.cu", []),
    ("lbm_staged.cu", []),
    ("lbm_batch.cu", []),
    ("lbm_forcing.cu", ["-fmad=false"]),
    ("lbm_particles.cu", ["-fmad=false"]),
    ("lbm_capi.cu", []),
    ("lbm_noalloc.cu", []),
    ("lbm_probe.cu", []),
    ("lbm_stats.cu", []),
    ("lbm_server.cu", []),
]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe is None:
        cand = Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300")
    return exe


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every unit (in parallel) and link the shared library."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "lbm.h"]
    exe = nvcc()
    procs = []
    objs = []
    for src, extra in UNITS:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [exe, *ARCH, *COMMON, *extra, "-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or _stale(LIB, objs):
        cudalib = Path(exe).resolve().parent.parent / "lib64"
        cmd = [exe, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcufft",
               "-Xlinker", "-rpath", "-Xlinker", str(cudalib)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
