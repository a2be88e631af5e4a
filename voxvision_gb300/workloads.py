"""Seeded synthetic volumes, cameras and query sets.

The reference measures nothing on public data for this path, so every
workload here is generated from a stated seed: voxel volumes as in a raw
dataset (voxel (i, j, k) sits at (i*vx, j*vy, k*vz), i outermost, as
src/voxtrees/datareader.c:51-74 lays them out), orbit cameras, and
incoherent ray / ball batches.  Integer randomness is splitmix64 so the same
seed gives the same bits on every host.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n outputs of splitmix64 started from `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """n float64 values in [0, 1) from the top 53 bits of splitmix64."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def gaussian(seed: int, n: int) -> np.ndarray:
    """n standard normal float64 values (Box-Muller over splitmix64)."""
    m = (n + 1) // 2
    u = uniform01(seed, 2 * m)
    u1 = np.maximum(u[:m], 1e-300)
    r = np.sqrt(-2.0 * np.log(u1))
    th = 2.0 * np.pi * u[m:]
    return np.concatenate([r * np.cos(th), r * np.sin(th)])[:n]


def texture32(seed: int = 7) -> np.ndarray:
    """The 32^3 u8 colour texture (stand-in for vn3d's noise, renderer.c:54-71)."""
    return (splitmix64(seed, 32 * 32 * 32) >> np.uint64(56)).astype(np.uint8)


def blobs_volume(n: int = 64, nblobs: int = 20, seed: int = 1, solid: float = 0.20) -> np.ndarray:
    """Sum of Gaussian blobs (sigma U[3,10], amplitude 255) + U[0,16] noise,
    thresholded at the (1-solid) quantile.  Returns a bool mask (n, n, n)."""
    u = uniform01(seed, nblobs * 4 + n * n * n)
    centres = u[: nblobs * 3].reshape(nblobs, 3) * n
    sigmas = 3.0 + 7.0 * u[nblobs * 3: nblobs * 4]
    noise = 16.0 * u[nblobs * 4:].reshape(n, n, n)
    ax = np.arange(n, dtype=np.float64)
    vol = noise.copy()
    for c, s in zip(centres, sigmas):
        gx = np.exp(-((ax - c[0]) ** 2) / (2 * s * s))
        gy = np.exp(-((ax - c[1]) ** 2) / (2 * s * s))
        gz = np.exp(-((ax - c[2]) ** 2) / (2 * s * s))
        vol += 255.0 * gx[:, None, None] * gy[None, :, None] * gz[None, None, :]
    q = np.quantile(vol, 1.0 - solid)
    return vol > q


def value_noise_u8(n: int, seed: int, spacing: int = 16) -> np.ndarray:
    """Trilinear-upsampled value noise in [0, 255] as uint8, float32 arithmetic."""
    m = n // spacing + 1
    lat = (splitmix64(seed, m * m * m) >> np.uint64(56)).astype(np.float32).reshape(m, m, m)
    t = (np.arange(n, dtype=np.float32) % spacing) / np.float32(spacing)
    i0 = np.arange(n) // spacing
    out = np.empty((n, n, n), dtype=np.uint8)
    for a in range(n):  # one slab at a time keeps memory small for 512^3
        ia, ta = i0[a], t[a]
        s0 = lat[ia] * (np.float32(1) - ta) + lat[ia + 1] * ta          # (m, m)
        s1 = s0[i0] * (np.float32(1) - t)[:, None] + s0[i0 + 1] * t[:, None]   # (n, m)
        s2 = s1[:, i0] * (np.float32(1) - t)[None, :] + s1[:, i0 + 1] * t[None, :]
        out[a] = np.clip(s2, 0, 255).astype(np.uint8)
    return out


def band_for_fraction(vol: np.ndarray, solid: float, centre: int = 128) -> tuple[int, int]:
    """Smallest band [lo, lo+w) around `centre` whose occupancy reaches `solid`."""
    hist = np.bincount(vol.ravel(), minlength=256).astype(np.int64)
    total = vol.size
    best = (centre, 1)
    for w in range(1, 256):
        lo = max(0, min(255 - w + 1, centre - w // 2))
        if hist[lo: lo + w].sum() >= solid * total:
            return lo, w
        best = (lo, w)
    return best


def noise_volume(n: int, seed: int, solid: float, spacing: int = 16) -> np.ndarray:
    vol = value_noise_u8(n, seed, spacing)
    lo, w = band_for_fraction(vol, solid)
    return (vol >= lo) & (vol < lo + w)


def voxels_from_mask(mask: np.ndarray, voxel=(1.0, 1.0, 1.0)) -> np.ndarray:
    """(k, 3) float32 voxel min-corners in datareader order (i outermost)."""
    idx = np.argwhere(mask)
    out = idx.astype(np.float32)
    out *= np.asarray(voxel, dtype=np.float32)[None, :]
    return np.ascontiguousarray(out)


def orbit_pose(frame: int, nframes: int, centre, radius: float, elevation_deg: float = 20.0):
    """Camera position for frame `frame` of an orbit around `centre`."""
    az = 2.0 * math.pi * frame / nframes
    el = math.radians(elevation_deg)
    c = np.asarray(centre, dtype=np.float64)
    pos = c + radius * np.array([math.cos(el) * math.cos(az), math.cos(el) * math.sin(az), math.sin(el)])
    return pos.astype(np.float32)


def incoherent_rays(n: int, lo: float, hi: float, seed: int):
    """Origins uniform in [lo, hi)^3, directions uniform on the sphere (float32)."""
    u = uniform01(seed, 3 * n).reshape(n, 3)
    origins = (lo + (hi - lo) * u).astype(np.float32)
    g = gaussian(seed + 0x5151, 3 * n).reshape(n, 3)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return np.ascontiguousarray(origins), np.ascontiguousarray(g.astype(np.float32))


def balls(n: int, lo: float, hi: float, rmin: float, rmax: float, seed: int):
    u = uniform01(seed, 4 * n)
    centres = (lo + (hi - lo) * u[: 3 * n]).reshape(n, 3).astype(np.float32)
    radii = (rmin + (rmax - rmin) * u[3 * n:]).astype(np.float32)
    return np.ascontiguousarray(centres), np.ascontiguousarray(radii)


RESOLUTIONS = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]
BATCH_TREES = [(64, 10, 0.05), (128, 11, 0.10), (256, 12, 0.15), (512, 13, 0.20)]


def batch_poses(n: int = 64, ntrees: int = 4, seed: int = 14):
    """n frame requests of the mixed-camera load: (tree index, (w, h),
    azimuth, elevation) with resolution and tree uniform, azimuth U[0, 2pi),
    elevation U[5, 45] degrees."""
    u = uniform01(seed, 4 * n).reshape(n, 4)
    out = []
    for i in range(n):
        ti = min(int(u[i, 0] * ntrees), ntrees - 1)
        ri = min(int(u[i, 1] * len(RESOLUTIONS)), len(RESOLUTIONS) - 1)
        az = 2.0 * math.pi * u[i, 2]
        el = 5.0 + 40.0 * u[i, 3]
        out.append((ti, RESOLUTIONS[ri], az, el))
    return out


def pose_position(centre, radius: float, az: float, el_deg: float) -> np.ndarray:
    el = math.radians(el_deg)
    c = np.asarray(centre, dtype=np.float64)
    return (c + radius * np.array([math.cos(el) * math.cos(az), math.cos(el) * math.sin(az),
                                   math.sin(el)])).astype(np.float32)
