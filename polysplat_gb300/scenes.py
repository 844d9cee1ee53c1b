"""Seeded synthetic Gaussian scenes and cameras for the five benchmark workloads.

The reference benchmarks trained INRIA scenes (Mip-NeRF 360, Tanks & Temples);
none are available offline, so seeded numpy PCG64 scenes with the stated
shapes and value distributions stand in for them.  Every scene is returned
in *raw* INRIA parameterisation (means, log-scales, w-first quaternions,
opacity logits, SH ``[P,16,3]``), exactly what a ``point_cloud.ply`` holds
(``csrc/pybind.cpp:12-20``); :func:`polysplat_gb300.rasterizer.Scene` turns
them into ``pos / shs / opacity / cov3d`` on the GPU.

Workloads (sizes and distributions):

* ``plain_100k_800x600`` (seed 0): N=100,000; means N(0, 2^2 I); log-scales
  N(-3.5, 0.5); quaternions normalised N(0, I4); opacity = sigmoid(N(0, 1.5));
  SH DC N(0, 0.5), higher orders N(0, 0.05); camera at (0,0,-8) looking at the
  origin, fx=fy=600, 800x600.
* ``plain_3m_1080p`` (seed 1): N=3,000,000; 90% from 64 clusters (centres
  U[-10,10]^3, per-axis sigma U[0.1, 2]), 10% on a radius-30 shell; log-scales
  Student-t(3, loc -4, scale 0.6); camera as above; 1920x1080, fx=fy=1400.
* ``city_20m_8k`` (seed 2): N=20,000,000; ground plane 200x200 with heights
  Exp(mean 8) plus 4,096 clusters of 2,000 points; log-scales N(-4.5, 0.7);
  7680x4320, fx=fy=5000.
* ``serve_mix`` (seed 3): resident scenes of 0.5/2/5/10 M Gaussians drawn as
  ``plain_3m_1080p``; 512 requests, Poisson arrivals at 240/s, scene uniform,
  resolution uniform over 720p/1080p/1440p/2160p, orbit radius U[6,12].
* ``diff_1m_8cam`` (seed 4): N=1,000,000 as ``plain_100k_800x600`` with means
  N(0, 3^2 I); 8 cameras at 1280x720 on a radius-10 orbit.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List

import numpy as np

SH_C0 = 0.28209479177387814


@dataclasses.dataclass
class RawScene:
    """Raw Gaussian parameters (float32, host memory)."""

    means: np.ndarray        # [P,3]
    log_scales: np.ndarray   # [P,3]
    quats: np.ndarray        # [P,4] (w, x, y, z), normalised
    opacity_logits: np.ndarray  # [P]
    shs: np.ndarray          # [P,16,3]

    @property
    def num(self) -> int:
        return int(self.means.shape[0])


@dataclasses.dataclass
class CameraSpec:
    """Pinhole camera in the INRIA ``cameras.json`` convention.

    ``rotation`` is camera-to-world (columns = right, down, forward in world
    coordinates); the rasterizer uses its transpose as world-to-view, which is
    what ``csrc/pybind.cpp:141-143`` does with the JSON rows.
    """

    width: int
    height: int
    position: np.ndarray  # [3]
    rotation: np.ndarray  # [3,3]
    fx: float
    fy: float
    id: int = 0
    img_name: str = "synthetic"

    def to_json(self) -> dict:
        return {
            "id": self.id,
            "img_name": self.img_name,
            "width": int(self.width),
            "height": int(self.height),
            "position": [float(v) for v in self.position],
            "rotation": [[float(v) for v in row] for row in self.rotation],
            "fx": float(self.fx),
            "fy": float(self.fy),
        }


def look_at(position, target, width, height, fx, fy, **kw) -> CameraSpec:
    """Camera at ``position`` looking at ``target`` with world up = -y (y down)."""
    pos = np.asarray(position, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - pos
    f /= np.linalg.norm(f)
    up = np.array([0.0, -1.0, 0.0])
    right = np.cross(f, up)
    n = np.linalg.norm(right)
    if n < 1e-9:  # looking straight up/down
        right = np.array([1.0, 0.0, 0.0])
    else:
        right /= n
    down = np.cross(f, right)
    rot = np.stack([right, down, f], axis=1)  # columns
    return CameraSpec(width, height, pos.astype(np.float32), rot.astype(np.float32), fx, fy, **kw)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _common_attrs(rng: np.random.Generator, n: int):
    q = rng.standard_normal((n, 4), dtype=np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    logits = rng.normal(0.0, 1.5, n).astype(np.float32)
    shs = np.empty((n, 16, 3), dtype=np.float32)
    shs[:, 0, :] = rng.normal(0.0, 0.5, (n, 3))
    shs[:, 1:, :] = rng.normal(0.0, 0.05, (n, 15, 3))
    return q.astype(np.float32), logits, shs


def scene_plain_small(n: int = 100_000, seed: int = 0, mean_sigma: float = 2.0) -> RawScene:
    rng = _rng(seed)
    means = rng.normal(0.0, mean_sigma, (n, 3)).astype(np.float32)
    log_scales = rng.normal(-3.5, 0.5, (n, 3)).astype(np.float32)
    q, logits, shs = _common_attrs(rng, n)
    return RawScene(means, log_scales, q, logits, shs)


def scene_clustered(n: int = 3_000_000, seed: int = 1) -> RawScene:
    rng = _rng(seed)
    n_cl = int(round(n * 0.9))
    n_sh = n - n_cl
    centres = rng.uniform(-10.0, 10.0, (64, 3))
    sig = rng.uniform(0.1, 2.0, (64, 3))
    which = rng.integers(0, 64, n_cl)
    cl = centres[which] + rng.standard_normal((n_cl, 3)) * sig[which]
    d = rng.standard_normal((n_sh, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    shell = 30.0 * d
    means = np.concatenate([cl, shell], axis=0).astype(np.float32)
    log_scales = (-4.0 + 0.6 * rng.standard_t(3, (n, 3))).astype(np.float32)
    q, logits, shs = _common_attrs(rng, n)
    return RawScene(means, log_scales, q, logits, shs)


def scene_needles(n: int = 200_000, seed: int = 5) -> RawScene:
    """Test scene of strongly anisotropic Gaussians: one axis up to e^7
    (about 1100) times the other two, random orientations, many of them
    large on screen.  Their conics are ill-conditioned, the hard case for the
    tile tests."""
    rng = _rng(seed)
    means = rng.normal(0.0, 3.0, (n, 3)).astype(np.float32)
    log_scales = np.empty((n, 3), np.float32)
    log_scales[:, 0] = rng.uniform(-2.5, 0.0, n)
    log_scales[:, 1:] = log_scales[:, :1] - rng.uniform(0.0, 7.0, (n, 2))
    q, logits, shs = _common_attrs(rng, n)
    return RawScene(means, log_scales, q, logits, shs)


def scene_city(n: int = 20_000_000, seed: int = 2, n_clusters: int = 4096, per_cluster: int = 2000) -> RawScene:
    rng = _rng(seed)
    n_cl = min(n, n_clusters * per_cluster)
    n_pl = n - n_cl
    plane = np.empty((n_pl, 3), dtype=np.float32)
    plane[:, 0] = rng.uniform(-100.0, 100.0, n_pl)
    plane[:, 2] = rng.uniform(-100.0, 100.0, n_pl)
    plane[:, 1] = -rng.exponential(8.0, n_pl)  # y is down: heights go to -y
    cc = np.empty((n_clusters, 3))
    cc[:, 0] = rng.uniform(-100.0, 100.0, n_clusters)
    cc[:, 2] = rng.uniform(-100.0, 100.0, n_clusters)
    cc[:, 1] = -rng.exponential(8.0, n_clusters)
    csig = rng.uniform(0.3, 1.5, n_clusters)
    which = np.repeat(np.arange(n_clusters), per_cluster)[:n_cl]
    cl = (cc[which] + rng.standard_normal((n_cl, 3)) * csig[which, None]).astype(np.float32)
    means = np.concatenate([plane, cl], axis=0)
    log_scales = rng.normal(-4.5, 0.7, (n, 3)).astype(np.float32)
    q, logits, shs = _common_attrs(rng, n)
    return RawScene(means, log_scales, q, logits, shs)


def camera_front(width: int, height: int, f: float) -> CameraSpec:
    """Camera at (0,0,-8), identity camera-to-world rotation (+z forward, y down)."""
    return CameraSpec(width, height, np.array([0.0, 0.0, -8.0], np.float32), np.eye(3, dtype=np.float32), f, f)


def camera_city() -> CameraSpec:
    return look_at([0.0, -25.0, -130.0], [0.0, -5.0, 0.0], 7680, 4320, 5000.0, 5000.0)


def orbit_camera(radius: float, azimuth: float, elevation: float, width: int, height: int, f: float,
                 centre=(0.0, 0.0, 0.0), **kw) -> CameraSpec:
    c = np.asarray(centre, dtype=np.float64)
    pos = c + radius * np.array([math.cos(elevation) * math.sin(azimuth),
                                 -math.sin(elevation),
                                 -math.cos(elevation) * math.cos(azimuth)])
    return look_at(pos, c, width, height, f, f, **kw)


# Named workloads -----------------------------------------------------------------

RESOLUTIONS = [(1280, 720), (1920, 1080), (2560, 1440), (3840, 2160)]


def focal_for(width: int) -> float:
    """Focal length giving the 1080p workload's horizontal field of view (fx=1400 at 1920)."""
    return 1400.0 * width / 1920.0


def workload(name: str):
    """Return (RawScene, [CameraSpec]) for a named plain-forward workload."""
    if name == "plain_100k_800x600":
        return scene_plain_small(), [camera_front(800, 600, 600.0)]
    if name == "plain_3m_1080p":
        return scene_clustered(), [camera_front(1920, 1080, 1400.0)]
    if name == "city_20m_8k":
        return scene_city(), [camera_city()]
    if name == "clustered_1m_1080p":  # a third-size plain_3m_1080p, for profiling captures
        return scene_clustered(1_000_000, seed=1), [camera_front(1920, 1080, 1400.0)]
    if name == "diff_1m_8cam":
        scene = scene_plain_small(1_000_000, seed=4, mean_sigma=3.0)
        cams = [orbit_camera(10.0, 2 * math.pi * k / 8, 0.0, 1280, 720, 900.0, id=k) for k in range(8)]
        return scene, cams
    raise KeyError(name)


@dataclasses.dataclass
class Request:
    arrival_s: float
    scene: int
    camera: CameraSpec


def serve_mix(num_requests: int = 512, rate_hz: float = 240.0, seed: int = 3,
              scene_sizes=(500_000, 2_000_000, 5_000_000, 10_000_000)):
    """Serving workload: resident scenes + a Poisson request stream."""
    rng = _rng(seed)
    scenes = [scene_clustered(n, seed=seed * 100 + i) for i, n in enumerate(scene_sizes)]
    t = 0.0
    reqs: List[Request] = []
    for k in range(num_requests):
        t += rng.exponential(1.0 / rate_hz)
        s = int(rng.integers(0, len(scenes)))
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        r = rng.uniform(6.0, 12.0)
        az = rng.uniform(0.0, 2 * math.pi)
        el = rng.uniform(-math.pi / 6, math.pi / 6)
        reqs.append(Request(t, s, orbit_camera(r, az, el, w, h, focal_for(w), id=k)))
    return scenes, reqs


def subsample(scene: RawScene, n: int, seed: int = 0) -> RawScene:
    """Deterministic subset of a scene (for small parity cases)."""
    if n >= scene.num:
        return scene
    idx = np.sort(_rng(seed).choice(scene.num, n, replace=False))
    return RawScene(scene.means[idx], scene.log_scales[idx], scene.quats[idx],
                    scene.opacity_logits[idx], scene.shs[idx])


def write_ply(path: str, scene: RawScene) -> None:
    """Write an INRIA-layout binary PLY (62 float32 per vertex, ``csrc/pybind.cpp:12-20``)."""
    n = scene.num
    rec = np.zeros((n, 62), dtype=np.float32)
    rec[:, 0:3] = scene.means
    # 3:6 normals (ignored)
    rec[:, 6:9] = scene.shs[:, 0, :]
    # f_rest is stored channel-major: 15 R coeffs, then 15 G, then 15 B
    rest = scene.shs[:, 1:, :]  # [P,15,3]
    rec[:, 9:54] = np.transpose(rest, (0, 2, 1)).reshape(n, 45)
    rec[:, 54] = scene.opacity_logits
    rec[:, 55:58] = scene.log_scales
    rec[:, 58:62] = scene.quats
    names = (["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
             + [f"f_rest_{i}" for i in range(45)] + ["opacity", "scale_0", "scale_1", "scale_2",
                                                     "rot_0", "rot_1", "rot_2", "rot_3"])
    header = "ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % n
    header += "".join(f"property float {nm}\n" for nm in names) + "end_header\n"
    with open(path, "wb") as f:
        f.write(header.encode("ascii"))
        f.write(rec.astype("<f4").tobytes())
