"""Seeded synthetic scenes: the stand-ins for the reference's benchmark meshes.

The reference publishes timings on scanned/production meshes (Sponza ...
Lucy) that are not available here; these generators produce meshes of the
same sizes with controlled distributions.  All use numpy's PCG64 with
recorded seeds and return float32 arrays ``[n, 9]`` (triangles v0, v1, v2)
in the byte layout of ``NXB::Triangle``.

* ``uniform_soup``   -- centroids U[0,1]^3, each vertex = centroid +
  U[-0.005, 0.005]^3 (65,536 triangles, seed 0, in the plain small config);
* ``displaced_sphere`` -- a (nu x nv) UV grid on the unit sphere, each quad
  split in two, radius 1 + sum_k (0.02/k) sin(a_k*theta + b_k*phi + psi_k)
  for k = 1..8 with integer a_k, b_k in [1, 64] and psi_k in [0, 2*pi)
  drawn once from the seed (2048 x 1024 -> 4,194,304 triangles);
* ``clustered``      -- centroids from a mixture of 256 anisotropic
  Gaussians (means U[0,1]^3, per-axis sigma log-U[0.001, 0.05], weights
  Dirichlet(1)); v0 = centroid, v1 = v0 + l1*d1, v2 = v0 + l2*d2 with
  random unit directions d and lengths lognormal(mu=-6, sigma=1)
  (12,582,912 triangles).
"""
from __future__ import annotations

import numpy as np

CHUNK = 1 << 20


def uniform_soup(n: int = 65536, seed: int = 0, spread: float = 0.005) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    v = c[:, None, :] + rng.uniform(-spread, spread, size=(n, 3, 3))
    return v.reshape(n, 9).astype(np.float32)


def displaced_sphere(nu: int = 2048, nv: int = 1024, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = rng.integers(1, 65, size=8)
    b = rng.integers(1, 65, size=8)
    psi = rng.uniform(0.0, 2.0 * np.pi, size=8)
    theta = np.linspace(0.0, np.pi, nv + 1)[:, None]
    phi = (2.0 * np.pi / nu) * np.arange(nu)[None, :]
    r = np.ones((nv + 1, nu))
    for k in range(8):
        r += (0.02 / (k + 1)) * np.sin(a[k] * theta + b[k] * phi + psi[k])
    st = np.sin(theta)
    verts = np.stack([r * st * np.cos(phi), r * st * np.sin(phi), r * np.cos(theta) * np.ones_like(phi)], axis=-1)
    verts = verts.astype(np.float32)
    j1 = (np.arange(nu) + 1) % nu
    v00 = verts[:-1, :]
    v10 = verts[1:, :]
    v11 = verts[1:, j1]
    v01 = verts[:-1, j1]
    t1 = np.concatenate([v00, v10, v11], axis=-1)
    t2 = np.concatenate([v00, v11, v01], axis=-1)
    tris = np.stack([t1, t2], axis=2)  # (nv, nu, 2, 9)
    return np.ascontiguousarray(tris.reshape(-1, 9))


def clustered(n: int = 12_582_912, seed: int = 2, components: int = 256) -> np.ndarray:
    rng = np.random.default_rng(seed)
    means = rng.random((components, 3))
    sigma = np.exp(rng.uniform(np.log(0.001), np.log(0.05), size=(components, 3)))
    weights = rng.dirichlet(np.ones(components))
    out = np.empty((n, 9), dtype=np.float32)
    children = np.random.SeedSequence(seed).spawn((n + CHUNK - 1) // CHUNK)
    for ci, start in enumerate(range(0, n, CHUNK)):
        m = min(CHUNK, n - start)
        r = np.random.default_rng(children[ci])
        comp = r.choice(components, size=m, p=weights)
        c = means[comp] + r.standard_normal((m, 3)) * sigma[comp]
        d1 = r.standard_normal((m, 3))
        d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
        d2 = r.standard_normal((m, 3))
        d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
        l1 = r.lognormal(-6.0, 1.0, size=(m, 1))
        l2 = r.lognormal(-6.0, 1.0, size=(m, 1))
        out[start:start + m, 0:3] = c
        out[start:start + m, 3:6] = c + l1 * d1
        out[start:start + m, 6:9] = c + l2 * d2
    return out


def batch_counts(meshes: int = 1024, seed: int = 3, lo: int = 256, hi: int = 262_144) -> np.ndarray:
    """Primitive counts of a batch: log-uniform in [lo, hi] (1024 meshes,
    about 38.7M triangles in expectation)."""
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size=meshes))).astype(np.int64).clip(lo, hi)


def batch_meshes(counts, seed: int = 3) -> np.ndarray:
    """Meshes end to end: each a uniform soup (centroids U[0,1]^3, vertex
    offsets U[-0.005, 0.005]^3) placed in its own box, origin U[-100, 100]^3
    and per-axis extent log-U[0.1, 10]."""
    rng = np.random.default_rng(seed + 1000)
    total = int(np.sum(counts))
    out = np.empty((total, 9), dtype=np.float32)
    at = 0
    for m, n in enumerate(counts):
        n = int(n)
        if n == 0:
            continue
        origin = rng.uniform(-100.0, 100.0, size=3)
        extent = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=3))
        soup = uniform_soup(n, seed=seed * 100_003 + m).reshape(n, 3, 3).astype(np.float64)
        out[at:at + n] = (origin + soup * extent).reshape(n, 9).astype(np.float32)
        at += n
    return out


def to_boxes(tris: np.ndarray) -> np.ndarray:
    """[n, 9] triangles -> [n, 6] boxes (NXB::AABB layout)."""
    v = tris.reshape(-1, 3, 3)
    return np.ascontiguousarray(np.concatenate([v.min(axis=1), v.max(axis=1)], axis=1).astype(np.float32))


def by_name(name: str) -> np.ndarray:
    """The named full-size workloads."""
    if name == "soup65k":
        return uniform_soup()
    if name == "sphere4m":
        return displaced_sphere()
    if name == "clustered12m":
        return clustered()
    if name == "clustered4m":
        return clustered(4_194_304)
    if name == "clustered28m":  # the served workload's injected build
        return clustered(28_311_552, seed=5)
    raise KeyError(name)
