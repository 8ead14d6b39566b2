"""Seeded synthetic particle frames for the benchmark and test workloads.

No public dataset is named for this path (the reference's example data lives in a separate
repository), so every workload is generated here from a fixed seed. Each generator returns a
``Frame``: float32 ``xyzr`` records (N x 4), the bounding box {left, bottom, back, right, top, front}
(MultiParticleDataCall's ObjectSpaceBBox, plugins/geometry_calls/include/geometry_calls/
MultiParticleDataCall.h) and the grid resolution the workload is quoted on.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Frame:
    xyzr: np.ndarray            # (N, 4) float32: x, y, z, radius
    bbox: tuple                 # (left, bottom, back, right, top, front)
    res: tuple                  # (sizex, sizey, sizez)
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.xyzr.shape[0])


def _box(lo, hi):
    return (float(lo[0]), float(lo[1]), float(lo[2]), float(hi[0]), float(hi[1]), float(hi[2]))


def uniform(n: int = 100_000, edge: float = 100.0, radius: float = 0.5, res: int = 128, seed: int = 1) -> Frame:
    """Uniform particles in [0, edge)^3 with one global radius (the small plain-method workload:
    100k particles, [0,100]^3, r = 0.5, 128^3 grid)."""
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(0.0, edge, size=(n, 3)).astype(np.float32)
    xyzr = np.empty((n, 4), np.float32)
    xyzr[:, :3] = xyz
    xyzr[:, 3] = np.float32(radius)
    return Frame(xyzr, _box((0, 0, 0), (edge, edge, edge)), (res, res, res), f"uniform_{n}",
                 dict(global_radius=radius))


def fcc_lattice(cells: int, spacing: float) -> np.ndarray:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], np.float64)
    g = np.arange(cells, dtype=np.float64)
    cz, cy, cx = np.meshgrid(g, g, g, indexing="ij")
    c = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1)
    return ((c[:, None, :] + base[None, :, :]).reshape(-1, 3) * spacing)


def lj_liquid(cells: int = 100, spacing: float = 1.12, jitter: float = 0.08, rmin: float = 0.4, rmax: float = 0.6,
              res: int = 256, seed: int = 2) -> Frame:
    """LJ-liquid-like frame: FCC lattice (4 sites per cell, `cells`^3 cells) jittered by N(0, jitter) per
    axis and wrapped into the periodic box [0, cells*spacing)^3, radii U[rmin, rmax]. The headline
    workload is cells=100 (4,000,000 particles) on a 256^3 grid."""
    rng = np.random.default_rng(seed)
    L = cells * spacing
    xyz = fcc_lattice(cells, spacing) + rng.normal(0.0, jitter, size=(4 * cells ** 3, 3))
    xyz = np.mod(xyz, L)
    n = xyz.shape[0]
    xyzr = np.empty((n, 4), np.float32)
    xyzr[:, :3] = xyz.astype(np.float32)
    # float rounding of mod() can produce exactly L; keep every particle inside the box
    xyzr[:, :3] = np.minimum(xyzr[:, :3], np.nextafter(np.float32(L), np.float32(0)))
    xyzr[:, 3] = rng.uniform(rmin, rmax, size=n).astype(np.float32)
    return Frame(xyzr, _box((0, 0, 0), (L, L, L)), (res, res, res), f"lj_liquid_{n}")


def blob_frame(rng: np.random.Generator, n: int, edge: float = 200.0, radius: float = 0.5) -> Frame:
    """One trajectory frame: a mixture of 1-8 isotropic Gaussian blobs (std U[2,10], centres U[0,edge]^3);
    the grid edge is matched to the occupied extent and taken from {64, 96, 128, 160, 192, 224, 256}."""
    k = int(rng.integers(1, 9))
    centres = rng.uniform(0.0, edge, size=(k, 3))
    stds = rng.uniform(2.0, 10.0, size=k)
    w = rng.dirichlet(np.ones(k))
    which = rng.choice(k, size=n, p=w)
    xyz = centres[which] + rng.normal(size=(n, 3)) * stds[which, None]
    xyzr = np.empty((n, 4), np.float32)
    xyzr[:, :3] = xyz.astype(np.float32)
    xyzr[:, 3] = np.float32(radius)
    lo = xyzr[:, :3].min(0)
    hi = xyzr[:, :3].max(0)
    ext = float((hi - lo).max())
    edges = np.array([64, 96, 128, 160, 192, 224, 256])
    res = int(edges[np.argmin(np.abs(edges - np.clip(ext / 0.5, 64, 256)))])
    return Frame(xyzr, _box(lo, hi), (res, res, res), f"blobs_{n}")


def trajectory(frames: int = 64, nmin: int = 50_000, nmax: int = 2_000_000, seed: int = 3) -> list[Frame]:
    """Batched trajectory: `frames` frames with particle counts log-uniform in [nmin, nmax]; frame f is
    generated from seed + f."""
    out = []
    for f in range(frames):
        rng = np.random.default_rng(seed + f)
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        out.append(blob_frame(rng, n))
    return out


def mixed_phase(n: int = 64_000_000, spacing: float = 1.12, jitter: float = 0.05, res: int = 512,
                seed: int = 5) -> Frame:
    """Large mixed-phase frame: half the particles an FCC crystal slab (spacing, jitter), half a uniform
    gas at 1/20 of the slab's number density; species radii 0.5 / 0.8 / 1.2 in ratio 6:3:1."""
    rng = np.random.default_rng(seed)
    half = n // 2
    rho = 4.0 / spacing ** 3
    # square slab cross-section of `side` cells, thickness chosen so the slab holds `half` sites
    side = int(np.ceil((half / 4.0) ** (1.0 / 3.0) * 1.6))
    thick = int(np.ceil(half / (4.0 * side * side)))
    g = np.arange(side, dtype=np.float64)
    t = np.arange(thick, dtype=np.float64)
    cz, cy, cx = np.meshgrid(t, g, g, indexing="ij")
    cells = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], np.float64)
    slab = ((cells[:, None, :] + base[None]).reshape(-1, 3) * spacing)[:half]
    slab += rng.normal(0.0, jitter, size=slab.shape)
    L = side * spacing
    gas_vol = (n - half) / (rho / 20.0)
    gas_h = gas_vol / (L * L)
    z0 = thick * spacing
    gas = np.column_stack([rng.uniform(0, L, n - half), rng.uniform(0, L, n - half),
                           rng.uniform(z0, z0 + gas_h, n - half)])
    xyz = np.concatenate([slab, gas]).astype(np.float32)
    species = rng.choice(3, size=n, p=[0.6, 0.3, 0.1])
    radii = np.array([0.5, 0.8, 1.2], np.float32)[species]
    xyzr = np.empty((n, 4), np.float32)
    xyzr[:, :3] = xyz
    xyzr[:, 3] = radii
    lo = xyz.min(0)
    hi = xyz.max(0)
    return Frame(xyzr, _box(lo, hi), (res, res, res), f"mixed_phase_{n}")


def random_normals(n: int, seed: int = 7) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v.astype(np.float32)


def gradient_normals(xyzr: np.ndarray, grid: np.ndarray, bbox, cyclic=True, seed: int = 11) -> np.ndarray:
    """Unit normals pointing down the local density gradient (outward from dense regions): -grad(rho)
    by central differences on the node grid (periodic when `cyclic`), trilinearly interpolated at each
    particle. Particles where the gradient vanishes get a seeded random direction."""
    g = np.asarray(grid, np.float32)
    sz, sy, sx = g.shape
    lo = np.array(bbox[:3], np.float64)
    hi = np.array(bbox[3:], np.float64)
    h = (hi - lo) / (np.array([sx, sy, sz]) - 1)
    grads = []
    for axis, ha in ((2, h[0]), (1, h[1]), (0, h[2])):
        if cyclic:
            d = (np.roll(g, -1, axis) - np.roll(g, 1, axis)) / (2 * ha)
        else:
            d = np.gradient(g, ha, axis=axis)
        grads.append(d.astype(np.float32))
    u = (xyzr[:, :3].astype(np.float64) - lo) / h
    u = np.clip(u, 0, np.array([sx, sy, sz]) - 1 - 1e-6)
    i0 = np.floor(u).astype(np.int64)
    f = (u - i0).astype(np.float32)
    i1 = np.minimum(i0 + 1, np.array([sx, sy, sz]) - 1)
    out = np.zeros((xyzr.shape[0], 3), np.float32)
    for c, G in enumerate(grads):
        acc = np.zeros(xyzr.shape[0], np.float32)
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * \
                        (f[:, 2] if dz else 1 - f[:, 2])
                    ix = i1[:, 0] if dx else i0[:, 0]
                    iy = i1[:, 1] if dy else i0[:, 1]
                    iz = i1[:, 2] if dz else i0[:, 2]
                    acc += w * G[iz, iy, ix]
        out[:, c] = -acc
    n = np.linalg.norm(out, axis=1, keepdims=True)
    bad = (n[:, 0] <= 1e-12) | ~np.isfinite(n[:, 0])
    if bad.any():
        out[bad] = random_normals(int(bad.sum()), seed)
        n[bad] = 1.0
    return (out / n).astype(np.float32)
