"""Seeded synthetic workloads (no dataset is involved anywhere).

- ring geometry: N_t transducers evenly spaced on a ring of radius
  0.95 x the half-width of an n x n image, every pair (i < j) one ray;
- hemisphere geometry: emitters and receivers interleaved on a seeded
  Fibonacci lattice of the lower hemisphere of radius 0.95 x the half-width of
  an n^3 volume, every emitter-receiver pair one ray;
- ellipse / ellipsoid phantoms; b = A x + Gaussian noise with
  sigma = level * ||A x|| / sqrt(m).

Coordinates are in voxel units: voxel (x, y, z) spans [x, x+1) x [y, y+1) x
[z, z+1); the integer coordinates used by Bresenham traversal are the voxels
containing the continuous positions.  Volumes are [z, x, y] arrays.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .api import Geometry
from .capi import TRAV_BRESENHAM, TRAV_SIDDON

GOLDEN_ANGLE = math.pi * (3.0 - math.sqrt(5.0))


def _int_coords(p, n):
    return np.clip(np.floor(p), 0, n - 1).astype(np.int32)


def ring_geometry(n_px: int = 64, n_trans: int = 128, radius_frac: float = 0.95,
                  traversal: int = TRAV_SIDDON) -> Geometry:
    """2D ring (dim_z = 1): all n_trans*(n_trans-1)/2 pairs i < j as rays."""
    c = n_px / 2.0
    R = radius_frac * n_px / 2.0
    th = 2.0 * np.pi * np.arange(n_trans) / n_trans
    px = c + R * np.cos(th)
    py = c + R * np.sin(th)
    pz = np.full(n_trans, 0.5)
    use = np.triu(np.ones((n_trans, n_trans), dtype=np.uint32), k=1).reshape(-1)
    ix, iy, iz = _int_coords(px, n_px), _int_coords(py, n_px), np.zeros(n_trans, np.int32)
    return Geometry(rv_x=n_px, rv_y=n_px, rv_z=1, x_emitters=ix, y_emitters=iy, z_emitters=iz,
                    x_receivers=ix, y_receivers=iy, z_receivers=iz, num_emitters=n_trans, num_receivers=n_trans,
                    numMPs=1, use_path=use, scale_factor=1.0, traversal=traversal,
                    pos=(px, py, pz, px, py, pz))


def hemisphere_geometry(n_vox: int = 128, n_em: int = 512, n_rc: int = 512, radius_frac: float = 0.95,
                        seed: int = 0, traversal: int = TRAV_SIDDON) -> Geometry:
    """3D bowl: n_em emitters and n_rc receivers on a Fibonacci lattice of the
    lower hemisphere (seeded rotation), all n_em*n_rc pairs as rays."""
    rng = np.random.default_rng(seed)
    N = n_em + n_rc
    k = np.arange(N)
    z = -(k + 0.5) / N
    r = np.sqrt(1.0 - z * z)
    phi = k * GOLDEN_ANGLE + rng.uniform(0.0, 2.0 * np.pi)
    c = n_vox / 2.0
    R = radius_frac * n_vox / 2.0
    P = np.stack([c + R * r * np.cos(phi), c + R * r * np.sin(phi), c + R * z], axis=1)
    # interleave: as many emitters as requested, evenly over the lattice
    order = np.argsort((np.arange(N) * n_em) % N, kind="stable") if n_em != n_rc else None
    if order is None:
        em, rc = P[0::2], P[1::2]
    else:
        em, rc = P[order[:n_em]], P[order[n_em:]]
    ie = [_int_coords(em[:, a], n_vox) for a in range(3)]
    ir = [_int_coords(rc[:, a], n_vox) for a in range(3)]
    return Geometry(rv_x=n_vox, rv_y=n_vox, rv_z=n_vox, x_emitters=ie[0], y_emitters=ie[1], z_emitters=ie[2],
                    x_receivers=ir[0], y_receivers=ir[1], z_receivers=ir[2], num_emitters=n_em,
                    num_receivers=n_rc, numMPs=1, use_path=None, scale_factor=1.0, traversal=traversal,
                    pos=(em[:, 0].copy(), em[:, 1].copy(), em[:, 2].copy(),
                         rc[:, 0].copy(), rc[:, 1].copy(), rc[:, 2].copy()))


def ellipse_phantom(n: int = 64, n_ell: int = 5, seed: int = 0, axes=(5.0, 25.0), values=(0.0, 1.0),
                    background: float = 0.0) -> np.ndarray:
    """[1, x, y] image of n_ell ellipses (later ones overwrite earlier ones)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.meshgrid(np.arange(n) + 0.5, np.arange(n) + 0.5, indexing="xy")
    img = np.full((n, n), background, dtype=np.float64)  # [x, y]
    X, Y = np.meshgrid(np.arange(n) + 0.5, np.arange(n) + 0.5, indexing="ij")
    for _ in range(n_ell):
        rr = 0.45 * n * math.sqrt(rng.uniform())
        ang = rng.uniform(0, 2 * np.pi)
        cx, cy = n / 2 + rr * math.cos(ang), n / 2 + rr * math.sin(ang)
        a, b = rng.uniform(*axes), rng.uniform(*axes)
        th = rng.uniform(0, np.pi)
        v = rng.uniform(*values)
        dx, dy = X - cx, Y - cy
        u = (dx * math.cos(th) + dy * math.sin(th)) / a
        w = (-dx * math.sin(th) + dy * math.cos(th)) / b
        img[u * u + w * w <= 1.0] = v
    del xx, yy
    return img[None, :, :].astype(np.float32)


def ellipsoid_phantom(n: int = 128, n_ell: int = 12, seed: int = 0, values=(0.9, 1.1),
                      background: float = 1.0, axes_frac=(0.06, 0.22)) -> np.ndarray:
    """[z, x, y] volume: n_ell random ellipsoids inside the scanned half-ball."""
    rng = np.random.default_rng(seed)
    vol = np.full((n, n, n), background, dtype=np.float32)
    c = n / 2.0
    R = 0.95 * n / 2.0
    g = np.arange(n) + 0.5
    for _ in range(n_ell):
        while True:
            p = rng.uniform(-1, 1, 3) * 0.6 * R
            if p[2] <= 0 and np.linalg.norm(p) <= 0.6 * R:
                break
        ctr = c + p  # (x, y, z)
        ax = rng.uniform(*axes_frac, 3) * n / 2.0 * 2.0
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        v = rng.uniform(*values)
        lo = np.maximum(0, np.floor(ctr - ax.max()).astype(int))
        hi = np.minimum(n, np.ceil(ctr + ax.max()).astype(int) + 1)
        Z, X, Y = np.meshgrid(g[lo[2]:hi[2]], g[lo[0]:hi[0]], g[lo[1]:hi[1]], indexing="ij")
        d = np.stack([X - ctr[0], Y - ctr[1], Z - ctr[2]], axis=-1) @ Q
        inside = ((d / ax) ** 2).sum(-1) <= 1.0
        sub = vol[lo[2]:hi[2], lo[0]:hi[0], lo[1]:hi[1]]
        sub[inside] = v
    return vol


def add_noise(Ax: np.ndarray, level: float, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 7919)
    Ax = np.asarray(Ax, dtype=np.float64)
    sigma = level * np.linalg.norm(Ax) / math.sqrt(max(Ax.size, 1))
    return (Ax + sigma * rng.standard_normal(Ax.shape)).astype(np.float32)


@dataclass
class Config:
    name: str
    dims: tuple          # (dim_y, dim_x, dim_z)
    opts: dict
    noise: float
    seed: int = 0


def config_2d(n_px=64, n_trans=128, seed=0) -> tuple[Config, Geometry, np.ndarray]:
    """The 2D plain-TVAL3 workload: 64x64, 128-transducer ring, 5 ellipses,
    1 % noise, anisotropic TV, mu 2^8, beta 2^5, tol 1e-4, maxit 300."""
    geo = ring_geometry(n_px, n_trans, traversal=TRAV_SIDDON)
    x = ellipse_phantom(n_px, 5, seed)
    cfg = Config("2d_ring", (n_px, n_px, 1),
                 dict(mu=2.0 ** 8, mu0=2.0 ** 8, beta=2.0 ** 5, beta0=2.0 ** 5, tol=1e-4, maxit=300, tv_type=0),
                 0.01, seed)
    return cfg, geo, x


def config_3d(n_vox=128, n_em=512, n_rc=512, seed=0) -> tuple[Config, Geometry, np.ndarray]:
    """The 3D plain-TVAL3 workload: 128^3, 512 x 512 Fibonacci-hemisphere rays,
    12 ellipsoids, 0.5 % noise, isotropic TV, mu 2^9, beta 2^6, tol 1e-4, maxit 200."""
    geo = hemisphere_geometry(n_vox, n_em, n_rc, seed=seed, traversal=TRAV_SIDDON)
    x = ellipsoid_phantom(n_vox, 12, seed)
    cfg = Config("3d_hemisphere", (n_vox, n_vox, n_vox),
                 dict(mu=2.0 ** 9, mu0=2.0 ** 9, beta=2.0 ** 6, beta0=2.0 ** 6, tol=1e-4, maxit=200, tv_type=1),
                 0.005, seed)
    return cfg, geo, x


def config_batched_2d(count: int = 64, seed: int = 0, side=(96, 256), n_trans=(128, 512)):
    """The batched-2D workload: `count` independent slices, each with its own
    side ~ U[96, 256] px and ring of N_t ~ U[128, 512] transducers (all
    N_t (N_t - 1) / 2 pairs as rays), the 2D phantom, noise and options of
    config_2d.  Returns a list of (Config, Geometry, phantom)."""
    rng = np.random.default_rng(seed + 104729)
    out = []
    for i in range(count):
        s = int(rng.integers(side[0], side[1] + 1))
        nt = int(rng.integers(n_trans[0], n_trans[1] + 1))
        out.append(config_2d(s, nt, seed + i))
    return out
