"""Build recipe of the in-tree CUDA library ``_build/libssp_gb300.so`` (sm_103a only).

Every ``csrc/*.cu`` is compiled separately (in parallel) as relocatable device code, host C++
sources with g++, and nvcc performs the device link into one shared library that exports the
C ABI declared in ``include/ssp_gb300.h``.  No CMake, no torch extension machinery.
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libssp_gb300.so"
# the benchmark's FP64 rate probe, kept out of the product library
PROBE_SRC = CSRC / "bench" / "fp64_probe.cu"
PROBE_LIB = BUILD / "libssp_fp64_probe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-rdc=true", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              f"-I{REPO / 'include'}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", f"-I{REPO / 'include'}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the sm_103a library cannot be built")


def _sources() -> tuple[list[Path], list[Path]]:
    return sorted(CSRC.glob("*.cu")), sorted(CSRC.glob("*.cpp"))


def _fingerprint() -> str:
    h = hashlib.sha256()
    cu, cpp = _sources()
    for p in [*cu, *cpp, *sorted(CSRC.glob("*.cuh")), PROBE_SRC, REPO / "include" / "ssp_gb300.h", Path(__file__)]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    stamp = BUILD / "fingerprint"
    fp = _fingerprint()
    if LIB.exists() and PROBE_LIB.exists() and not force and stamp.exists() and stamp.read_text() == fp:
        return LIB
    nvcc = _nvcc()
    cu, cpp = _sources()
    jobs = []
    for src in cu:
        obj = BUILD / (src.stem + ".o")
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-dc", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD / (src.stem + ".cpp.o")
        jobs.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {cmd[-3]}")
        return cmd[-1]

    probe_tmp = BUILD / (PROBE_LIB.name + ".tmp")
    probe_job = [nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-shared", str(PROBE_SRC),
                 "-o", str(probe_tmp)]
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs) + 1, os.cpu_count() or 4))) as ex:
        probe_done = ex.submit(run, probe_job)
        objs = list(ex.map(run, jobs))
        probe_done.result()
    probe_tmp.replace(PROBE_LIB)
    tmp = BUILD / (LIB.name + ".tmp")
    link = [nvcc, *ARCH, "-shared", "-rdc=true", "-Xcompiler", "-fPIC", *objs, "-o", str(tmp), "-lcudart"]
    run(link)
    tmp.replace(LIB)
    stamp.write_text(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
