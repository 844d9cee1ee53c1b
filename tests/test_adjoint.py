"""The preprocess adjoint (polysplat_gb300/csrc/adjoint.h) in double against
central differences of the same forward: every parameter of random
Gaussians, including coordinates clamped to the 1.3 tan(fov) cone and colour
channels clamped at 0.  Bar: relative error <= 1e-6 (of the largest
gradient of the case)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    out = str(tmp_path_factory.mktemp("adj") / "libadj.so")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(HERE, "adjoint_shim.cpp"),
                           "-o", out])
    L = ctypes.CDLL(out)
    P = ctypes.c_void_p
    L.adj_forward.argtypes = [P] * 8
    L.adj_backward.argtypes = [P] * 8
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _camera(W=640, H=480, f=500.0, pos=(0.0, 0.0, -8.0)):
    """View (identity rotation) and projection, column-major, as the
    library builds them for a camera looking down +z."""
    view = np.eye(4)
    view[3, :3] = -np.asarray(pos)  # translation in the last column of the column-major array
    zf, zn = 100.0, 0.01
    tanx, tany = W / (2 * f), H / (2 * f)
    top, right = tany * zn, tanx * zn
    P = np.zeros((4, 4))
    P[0, 0] = 2 * zn / (2 * right)
    P[1, 1] = 2 * zn / (2 * top)
    P[3, 2] = 1.0
    P[2, 2] = zf / (zf - zn)
    P[2, 3] = -(zf * zn) / (zf - zn)
    proj_rowmajor = P @ view.T  # world -> clip
    proj = proj_rowmajor.T.copy()  # column-major storage
    return (view.copy(), proj, np.asarray(pos, float), np.array([f, f, tanx, tany]), np.array([W, H], np.int32))


def _fwd(L, params, cam):
    out = np.zeros(10)
    flags = np.zeros(5, np.int32)
    L.adj_forward(_p(params), *[_p(c) for c in cam], _p(out), _p(flags))
    return out, flags


def _check(L, params, cam, rng):
    g = rng.normal(size=9)
    grad = np.zeros(59)
    L.adj_backward(_p(params), *[_p(c) for c in cam], _p(g), _p(grad))
    num = np.zeros(59)
    for k in range(59):
        h = 1e-6 * max(1.0, abs(params[k]))
        pp, pm = params.copy(), params.copy()
        pp[k] += h
        pm[k] -= h
        op, fp = _fwd(L, pp, cam)
        om, fm = _fwd(L, pm, cam)
        assert (fp == fm).all(), "a clamp flipped inside the difference step"
        num[k] = (g @ op[:9] - g @ om[:9]) / (2 * h)
    scale = max(1e-12, np.abs(num).max())
    err = np.abs(grad - num).max() / scale
    assert err <= 1e-6, (err, np.argmax(np.abs(grad - num)))
    return _fwd(L, params, cam)[1]


def _params(rng, m, sh_scale=0.3):
    q = rng.normal(size=4)
    return np.concatenate([np.asarray(m, float), rng.normal(-1.0, 0.4, 3), q, [rng.normal(0, 1.5)],
                           rng.normal(0, sh_scale, 48)])


def test_adjoint_matches_finite_differences(shim):
    rng = np.random.default_rng(0)
    cam = _camera()
    seen = {"clamp_x": False, "clamp_y": False, "clamp_rgb": False}
    for k in range(40):
        m = rng.normal(0, 1.5, 3)
        if k % 5 == 0:
            m = [rng.choice([-1, 1]) * rng.uniform(8, 15), rng.normal(0, 1), rng.uniform(-2, 2)]  # outside x cone
        if k % 7 == 0:
            m = [rng.normal(0, 1), rng.choice([-1, 1]) * rng.uniform(8, 15), rng.uniform(-2, 2)]  # outside y cone
        params = _params(rng, m, sh_scale=0.8 if k % 3 == 0 else 0.2)
        flags = _check(shim, params, cam, rng)
        seen["clamp_x"] |= bool(flags[0])
        seen["clamp_y"] |= bool(flags[1])
        seen["clamp_rgb"] |= bool(flags[2:].any())
    assert all(seen.values()), seen  # every clamp branch was exercised


def test_adjoint_forward_matches_oracle(shim):
    """The header's forward reproduces the preprocess (the FP64 oracle, which
    is pinned to the reference) for a real camera: the adjoint differentiates
    the function the library evaluates."""
    from oracle import oracle as O
    from polysplat_gb300 import scenes
    from polysplat_gb300._lib import lib

    raw = scenes.scene_plain_small(2000, seed=5)
    cam = scenes.orbit_camera(7.0, 0.6, 0.2, 640, 480, scenes.focal_for(640))
    op, cov = O.scene_transform(raw.log_scales, raw.quats, raw.opacity_logits)
    pre = O.preprocess(raw.means, raw.shs, op, cov, cam.width, cam.height, cam.position, cam.rotation, cam.fx, cam.fy)
    view = (ctypes.c_float * 16)()
    proj = (ctypes.c_float * 16)()
    pos = (ctypes.c_float * 3)(*[float(v) for v in cam.position])
    rot = (ctypes.c_float * 9)(*[float(v) for v in np.asarray(cam.rotation).reshape(-1)])
    lib().gsr_camera_matrices(cam.width, cam.height, pos, rot, cam.fx, cam.fy, 100.0, 0.01, view, proj)
    c = (np.array(view[:], float), np.array(proj[:], float), np.asarray(cam.position, float),
         np.array([cam.fx, cam.fy, cam.width / (2 * cam.fx), cam.height / (2 * cam.fy)]),
         np.array([cam.width, cam.height], np.int32))
    idx = np.flatnonzero(pre["emitted"])[:300]
    assert idx.size > 100
    for i in idx:
        params = np.concatenate([raw.means[i], raw.log_scales[i], raw.quats[i], [raw.opacity_logits[i]],
                                 raw.shs[i].reshape(-1)]).astype(float)
        out, _ = _fwd(shim, params, c)
        np.testing.assert_allclose(out[0:2], pre["xy"][i], rtol=1e-5, atol=2e-3)
        np.testing.assert_allclose(out[2:6], pre["con"][i], rtol=2e-3, atol=1e-6)
        np.testing.assert_allclose(out[6:9], pre["rgbd"][i, :3], rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(out[9], pre["rgbd"][i, 3], rtol=1e-5)
