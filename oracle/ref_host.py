"""Recipe for the reference's host-side functions -- TEST INFRASTRUCTURE.

Builds two small shared libraries under ``oracle/_ref/`` (git-ignored) from
the reference's sources where they lie (``GSR_REFERENCE_DIR``, default
``/root/reference``; read-only):

* ``libref_host_cam.so`` -- ``oracle/ref_host_cam.cu`` includes the reference's
  ``csrc/cuda_rasterizer/preprocess.cu`` and exports its host functions
  getViewMatrix / getProjectionMatrix (preprocess.cu:643-671);
* ``libref_host_ply.so`` -- ``oracle/ref_host_ply.cpp`` includes the
  reference's ``csrc/pybind.cpp`` (with libtorch, as its own build does) and
  exports its loadPly_torch / computeCov3D (pybind.cpp:22-120).  The
  bindings' other functions call the reference's CUDA launchers, which are
  not needed here: those symbols are bound to stubs that abort.

Flags follow the reference's setup.py:20-21 (host: -O3 -DNDEBUG -std=c++17).
The libraries run on the host only and are used by
``tests/golden/make_host_golden.py`` to write the committed fixture
``tests/golden/host_reference.npz``; nothing here runs on the GPU host.
"""
from __future__ import annotations

import ctypes
import os
import re
import shutil
import subprocess
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("GSR_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
CAM_LIB = os.path.join(OUT, "libref_host_cam.so")
PLY_LIB = os.path.join(OUT, "libref_host_ply.so")
CXX_FLAGS = ["-O3", "-DNDEBUG", "-std=c++17", "-fPIC"]


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _cuda_home():
    return os.path.dirname(os.path.dirname(_nvcc()))


def available() -> bool:
    return os.path.isdir(os.path.join(REF, "csrc"))


def build_cam(force: bool = False) -> str:
    src = os.path.join(HERE, "ref_host_cam.cu")
    if not force and os.path.exists(CAM_LIB) and os.path.getmtime(CAM_LIB) >= os.path.getmtime(src):
        return CAM_LIB
    os.makedirs(OUT, exist_ok=True)
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler",
           "-fPIC,-O3,-DNDEBUG", "-shared", "-I" + os.path.join(REF, "csrc"), src, "-o", CAM_LIB]
    subprocess.check_call(cmd)
    return CAM_LIB


def _stubs(obj: str) -> str:
    """A C source defining, as aborting stubs, the reference's own functions
    that the bindings object calls but that live in its CUDA sources."""
    nm = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout
    names = sorted({m.group(1) for m in re.finditer(r"\bU (_ZN9polysplat\S+)", nm)})
    lines = ["#include <stdlib.h>"]
    for i, n in enumerate(names):
        lines.append('void ref_stub_%d(void) __asm__("%s");' % (i, n))
        lines.append("void ref_stub_%d(void) { abort(); }" % i)
    return "\n".join(lines) + "\n"


def build_ply(force: bool = False) -> str:
    src = os.path.join(HERE, "ref_host_ply.cpp")
    if not force and os.path.exists(PLY_LIB) and os.path.getmtime(PLY_LIB) >= os.path.getmtime(src):
        return PLY_LIB
    import torch
    from torch.utils import cpp_extension

    os.makedirs(OUT, exist_ok=True)
    abi = "-D_GLIBCXX_USE_CXX11_ABI=%d" % int(torch._C._GLIBCXX_USE_CXX11_ABI)
    incs = ["-I" + p for p in cpp_extension.include_paths()] + [
        "-I" + sysconfig.get_paths()["include"], "-I" + os.path.join(_cuda_home(), "include"),
        "-I" + os.path.join(REF, "csrc")]
    obj = os.path.join(OUT, "ref_host_ply.o")
    subprocess.check_call(["g++"] + CXX_FLAGS + [abi, "-DTORCH_EXTENSION_NAME=ref_host_ply",
                                                 "-DTORCH_API_INCLUDE_EXTENSION_H"] + incs + ["-c", src, "-o", obj])
    stub_c = os.path.join(OUT, "ref_host_stubs.c")
    with open(stub_c, "w") as f:
        f.write(_stubs(obj))
    stub_o = os.path.join(OUT, "ref_host_stubs.o")
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-c", stub_c, "-o", stub_o])
    tlib = os.path.join(os.path.dirname(torch.__file__), "lib")
    subprocess.check_call(["g++", "-shared", obj, stub_o, "-o", PLY_LIB, "-L" + tlib, "-lc10", "-ltorch",
                           "-ltorch_cpu", "-ltorch_python", "-Wl,-rpath," + tlib,
                           "-L" + os.path.join(_cuda_home(), "lib64"), "-lcudart"])
    return PLY_LIB


def camera_matrices(width, height, pos, rot, fx, fy, zfar=100.0, znear=0.01):
    """(view, proj), column-major float32[16], from the reference's own host code."""
    import numpy as np

    L = ctypes.CDLL(build_cam())
    f = (ctypes.c_float * 16)
    view, proj = f(), f()
    fp = ctypes.POINTER(ctypes.c_float)
    L.ref_camera_matrices.argtypes = [ctypes.c_int, ctypes.c_int, fp, fp, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_float, fp, fp]
    p = np.ascontiguousarray(pos, dtype=np.float32).reshape(3)
    r = np.ascontiguousarray(rot, dtype=np.float32).reshape(9)
    L.ref_camera_matrices(int(width), int(height), p.ctypes.data_as(fp), r.ctypes.data_as(fp), float(fx), float(fy),
                          float(zfar), float(znear), view, proj)
    return np.array(view, dtype=np.float32), np.array(proj, dtype=np.float32)


def load_ply(path: str, n: int):
    """(pos [n,3], shs [n,48], opacity [n], cov3d [n,6]) from the reference's loadPly_torch."""
    import numpy as np

    import torch  # noqa: F401  (loads libtorch into the process before the library)

    L = ctypes.CDLL(build_ply())
    fp = ctypes.POINTER(ctypes.c_float)
    L.ref_load_ply.argtypes = [ctypes.c_char_p, ctypes.c_int, fp, fp, fp, fp]
    L.ref_load_ply.restype = ctypes.c_int
    pos = np.zeros((n, 3), np.float32)
    shs = np.zeros((n, 48), np.float32)
    op = np.zeros(n, np.float32)
    cov = np.zeros((n, 6), np.float32)
    got = L.ref_load_ply(path.encode(), n, pos.ctypes.data_as(fp), shs.ctypes.data_as(fp), op.ctypes.data_as(fp),
                         cov.ctypes.data_as(fp))
    if got != n:
        raise RuntimeError("reference loadPly returned %d vertices, expected %d" % (got, n))
    return pos, shs, op, cov


if __name__ == "__main__":
    print(build_cam(force=True), build_ply(force=True))
