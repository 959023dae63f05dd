"""Build recipe for the in-tree CUDA library ``liblightprop2d_gb300.so``.

Compiles every translation unit under ``csrc/`` for sm_103a with nvcc, in
parallel, and links one shared library next to this file.  No CMake, no
torch extension: the library exports a plain C ABI
(``include/lightprop2d_gb300.h``) that Python reaches through ctypes.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB_NAME = "liblightprop2d_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build the backend")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _fingerprint(extra_flags=()) -> str:
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            with open(os.path.join(d, f), "rb") as fh:
                h.update(f.encode() + fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + list(extra_flags)).encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False, jobs: int | None = None,
          extra_flags: list[str] | None = None) -> str:
    """Compile (if stale) and return the path of the shared library.

    ``extra_flags`` (e.g. ``-DLP_MIN_BLOCKS=3``) select a tuning variant; the
    stamp records them, so a later default build recompiles."""
    fp = _fingerprint(extra_flags or ())
    stamp = os.path.join(BUILD, "stamp")
    if (not force and os.path.exists(LIB_PATH) and os.path.exists(stamp)
            and open(stamp).read() == fp):
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, *flags, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{p.stderr}")
        if verbose and p.stderr:
            sys.stderr.write(p.stderr)
        return obj

    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp_lib = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp_lib, *objs, "-Xcompiler", "-fPIC"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stderr}")
    os.replace(tmp_lib, LIB_PATH)
    with open(stamp, "w") as fh:
        fh.write(fp)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
