"""Recipe for the reference-kernel runner -- TEST INFRASTRUCTURE.

Where the reference sources are present (``GSR_REFERENCE_DIR``, default
``/root/reference``; read-only), its
``csrc/cuda_rasterizer/preprocess.cu`` and ``render.cu`` are compiled exactly
as they lie, with the reference's own nvcc flags (setup.py:20) plus the
sm_103a target, into device images under ``oracle/_ref/`` (git-ignored; the
GPU host only receives these prebuilt images).  The reference's sort.cu is
not compiled: it does not build against CUDA 13's CCCL, and its contract
(CUB's stable radix sort) is reproduced exactly by the oracle.

``refrun.cpp`` (this project's launcher) is compiled wherever this runs.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("GSR_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
RUNNER = os.path.join(HERE, "_build", "librefrun.so")
REF_NVCC_FLAGS = ["-O3", "--use_fast_math", "--extra-device-vectorization", "-Xptxas=-O3", "-std=c++17"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_cubins(force: bool = False) -> bool:
    src_dir = os.path.join(REF, "csrc", "cuda_rasterizer")
    if not os.path.isdir(src_dir):
        return all(os.path.exists(os.path.join(OUT, f)) for f in ("preprocess.cubin", "render.cubin"))
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for name in ("preprocess", "render"):
        out = os.path.join(OUT, name + ".cubin")
        src = os.path.join(src_dir, name + ".cu")
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        cmd = [_nvcc()] + ARCH + REF_NVCC_FLAGS + ["-I" + os.path.join(REF, "csrc"), "-cubin", src, "-o", out]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE))
    ok = True
    for p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            ok = False
            print("reference cubin build failed:", err.decode(errors="replace")[-2000:])
    return ok


def build_runner(force: bool = False) -> str:
    src = os.path.join(HERE, "refrun.cu")
    os.makedirs(os.path.dirname(RUNNER), exist_ok=True)
    if force or not os.path.exists(RUNNER) or os.path.getmtime(RUNNER) < os.path.getmtime(src):
        cuda = os.path.dirname(os.path.dirname(_nvcc()))
        tmp = RUNNER + ".tmp%d" % os.getpid()
        subprocess.check_call([_nvcc()] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                                                  "-cudart", "shared", src, "-o", tmp,
                                                  "-L" + os.path.join(cuda, "lib64", "stubs"), "-lcuda"])
        os.replace(tmp, RUNNER)
    return RUNNER


def build(force: bool = False):
    have = build_cubins(force)
    build_runner(force)
    return have


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv))
