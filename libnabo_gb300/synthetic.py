"""Seeded synthetic workloads for the kNN benchmarks and parity tests.

No public dataset is named for this path, so these generators stand in for
real clouds with the stated shapes, sizes and value distributions:

* ``uniform``       n points uniform in [0, 1]^d (the 10k-point CPU-runnable
                    case and the 1M-point / 1M-query uniform case).
* ``lidar_scan``    a 64-beam spinning lidar (elevations -25..+15 degrees)
                    over a ground plane at z = -1.7 m and 20 random
                    axis-aligned boxes 1-10 m in size within 60 m; ranges are
                    ray hits plus N(0, 0.02 m) noise. 25,000 azimuth steps
                    give about 1.15 M returns (the 1.15 M-point scan);
                    ``n_azimuth=1800`` gives the 115 k-ray scan.
* ``lidar_queries`` the scan after a random 2-degree rotation and a 0.1 m
                    translation.
* ``gaussian_blobs`` mixture of anisotropic Gaussian blobs (batched clouds).
* ``clusters``      mixture of isotropic Gaussian clusters in d dimensions
                    with log-uniform sigma (higher-dimensional case).
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 1234


def uniform(n: int, d: int = 3, seed: int = SEED_BASE, dtype=np.float32) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.random((n, d), dtype=np.float64).astype(dtype)


def _boxes(rng, count=20, within=60.0, size=(1.0, 10.0), ground=-1.7):
    lo = np.empty((count, 3))
    hi = np.empty((count, 3))
    for b in range(count):
        ext = rng.uniform(size[0], size[1], 3)
        # centre within `within` metres horizontally, resting on the ground,
        # and not enclosing the sensor at the origin
        while True:
            c = rng.uniform(-within, within, 2)
            if np.hypot(*c) > 3.0 + 0.5 * np.hypot(ext[0], ext[1]):
                break
        lo[b] = [c[0] - ext[0] / 2, c[1] - ext[1] / 2, ground]
        hi[b] = [c[0] + ext[0] / 2, c[1] + ext[1] / 2, ground + ext[2]]
    return lo, hi


def lidar_scan(seed: int = SEED_BASE + 1, n_azimuth: int = 25000, beams: int = 64, elev_deg=(-25.0, 15.0),
               ground: float = -1.7, n_boxes: int = 20, noise: float = 0.02, max_range: float = 120.0,
               dtype=np.float32, noise_seed: int | None = None) -> np.ndarray:
    """Returns an (n, 3) cloud of ray returns (rays that hit nothing are dropped).
    ``noise_seed`` draws the range noise from its own generator: the same
    scene scanned again (another frame of a static scene)."""
    rng = np.random.default_rng(seed)
    lo, hi = _boxes(rng, n_boxes, ground=ground)
    if noise_seed is not None:
        rng = np.random.default_rng(noise_seed)
    elev = np.deg2rad(np.linspace(elev_deg[0], elev_deg[1], beams))
    az = np.linspace(0.0, 2.0 * np.pi, n_azimuth, endpoint=False)
    out = []
    # one azimuth block at a time keeps the temporaries small
    block = 2000
    for a0 in range(0, n_azimuth, block):
        a = az[a0:a0 + block]
        ce, se = np.cos(elev)[None, :], np.sin(elev)[None, :]
        dx = (np.cos(a)[:, None] * ce).reshape(-1)
        dy = (np.sin(a)[:, None] * ce).reshape(-1)
        dz = np.broadcast_to(se, (a.shape[0], beams)).reshape(-1)
        t = np.full(dx.shape, np.inf)
        down = dz < 0
        t[down] = ground / dz[down]
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / np.stack([dx, dy, dz], axis=1)
            for b in range(n_boxes):
                t1 = lo[b][None, :] * inv
                t2 = hi[b][None, :] * inv
                tmin = np.nanmax(np.minimum(t1, t2), axis=1)
                tmax = np.nanmin(np.maximum(t1, t2), axis=1)
                hit = (tmax >= np.maximum(tmin, 0.0)) & (tmin > 0)
                t = np.where(hit & (tmin < t), tmin, t)
        ok = np.isfinite(t) & (t < max_range)
        r = t[ok] + rng.normal(0.0, noise, ok.sum())
        out.append(np.stack([dx[ok] * r, dy[ok] * r, dz[ok] * r], axis=1))
    return np.concatenate(out).astype(dtype)


def lidar_queries(cloud: np.ndarray, seed: int = SEED_BASE + 1, angle_deg: float = 2.0, shift: float = 0.1):
    """The cloud after a random rotation by `angle_deg` and a `shift` translation."""
    rng = np.random.default_rng(seed + 1000)
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    th = np.deg2rad(angle_deg)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * (K @ K)
    tvec = rng.normal(size=3)
    tvec *= shift / np.linalg.norm(tvec)
    q = cloud.astype(np.float64) @ R.T + tvec
    return q.astype(cloud.dtype)


def gaussian_blobs(n: int, seed: int, blobs: int = 8, sigma=(0.05, 2.0), spread: float = 10.0,
                   dtype=np.float32) -> np.ndarray:
    """Mixture of `blobs` anisotropic Gaussians with per-axis sigma in `sigma`."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-spread, spread, (blobs, 3))
    sig = rng.uniform(sigma[0], sigma[1], (blobs, 3))
    rot = []
    for _ in range(blobs):
        qm, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        rot.append(qm)
    lab = rng.integers(0, blobs, n)
    z = rng.normal(size=(n, 3)) * sig[lab]
    pts = np.einsum("nij,nj->ni", np.stack(rot)[lab], z) + centres[lab]
    return pts.astype(dtype)


def clusters(n: int, d: int, seed: int, count: int = 32, sigma=(0.01, 1.0), spread: float = 5.0,
             dtype=np.float32, centres: np.ndarray | None = None, sigmas: np.ndarray | None = None):
    """Mixture of `count` isotropic Gaussian clusters with log-uniform sigma."""
    rng = np.random.default_rng(seed)
    if centres is None:
        centres = rng.uniform(-spread, spread, (count, d))
    if sigmas is None:
        sigmas = np.exp(rng.uniform(np.log(sigma[0]), np.log(sigma[1]), count))
    lab = rng.integers(0, count, n)
    pts = centres[lab] + rng.normal(size=(n, d)) * sigmas[lab][:, None]
    return pts.astype(dtype), centres, sigmas


def log_uniform_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
