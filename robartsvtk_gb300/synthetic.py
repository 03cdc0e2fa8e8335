"""Seeded synthetic HMF workloads.

The reference ships no data and no benchmark inputs; these generators build
the phantoms, data terms and smoothness images of the benchmark workloads
(volume size, label tree, noise level, smoothness weights, iteration count)
from a seed, with numpy.  All volumes are float32 [VZ, VY, VX].

Data terms are Gaussian negative log-likelihoods of the noisy intensity under
each class mean, made non-negative (the reference rejects negative costs,
vtkHierarchicalMaxFlowSegmentation.cxx:434-438).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    dims: tuple           # (VX, VY, VZ)
    parent: list          # parent id per vertex, -1 for the root
    data: dict            # leaf vertex -> float32 [VZ, VY, VX]
    smooth: dict = field(default_factory=dict)   # vertex -> float32 image (may share objects)
    alpha: dict = field(default_factory=dict)    # vertex -> smoothness weight
    iterations: int = 100
    step: float = 0.1
    cc: float = 0.25
    truth: np.ndarray | None = None             # ground-truth class per voxel (leaf index)

    @property
    def nvox(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    @property
    def leaves(self) -> list:
        kids = {v: [] for v in range(len(self.parent))}
        root = None
        for v, p in enumerate(self.parent):
            if p < 0:
                root = v
            else:
                kids[p].append(v)
        out, stack = [], [root]
        while stack:
            v = stack.pop()
            if not kids[v]:
                out.append(v)
            stack.extend(reversed(kids[v]))
        return out

    @property
    def n_nonroot(self) -> int:
        return len(self.parent) - 1

    @property
    def n_smooth_images(self) -> int:
        return len({id(s) for s in self.smooth.values()})


def _ellipsoid_labels(shape_zyx, n, rng, rmin, rmax, labels=None):
    vz, vy, vx = shape_zyx
    lab = np.zeros(shape_zyx, dtype=np.int32)
    z = np.arange(vz, dtype=np.float32)[:, None, None]
    y = np.arange(vy, dtype=np.float32)[None, :, None]
    x = np.arange(vx, dtype=np.float32)[None, None, :]
    for k in range(n):
        c = rng.uniform(0, 1, size=3) * np.array([vx, vy, vz])
        r = rng.uniform(rmin, rmax, size=3)
        inside = ((x - c[0]) / r[0]) ** 2 + ((y - c[1]) / r[1]) ** 2 + ((z - c[2]) / r[2]) ** 2 <= 1.0
        lab[inside] = k if labels is None else labels[k]
    return lab


def _nll(intensity, means, sigma, clamp_hi=None, shift_nonneg=True):
    out = []
    for mu in means:
        d = 0.5 * ((intensity - np.float32(mu)) / np.float32(sigma)) ** 2
        if not shift_nonneg:
            d = d + np.float32(np.log(sigma * np.sqrt(2 * np.pi)))
            d = np.maximum(d, 0)
        if clamp_hi is not None:
            d = np.minimum(d, np.float32(clamp_hi))
        out.append(np.ascontiguousarray(d, dtype=np.float32))
    return out


def _grad_smoothness(intensity, scale, denom):
    gz, gy, gx = np.gradient(intensity.astype(np.float32))
    g2 = gx * gx + gy * gy + gz * gz
    return np.ascontiguousarray(np.float32(scale) * np.exp(-g2 / np.float32(denom)), dtype=np.float32)


def boxes_flat3(seed=0, size=64, iterations=200) -> Workload:
    """64^3, background 0.2 plus two boxes 0.5 / 0.8 from seeded corners,
    sigma 0.08, flat tree of 3 leaves, D = clamp(-log N(I; mu, 0.08^2), 0, 20),
    constant alpha 0.1."""
    rng = np.random.default_rng(seed)
    n = size
    truth = np.zeros((n, n, n), dtype=np.int32)
    for k in (1, 2):
        lo = rng.integers(0, n // 2, size=3)
        hi = lo + rng.integers(n // 4, n // 2, size=3)
        truth[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = k
    means = [0.2, 0.5, 0.8]
    img = np.array(means, dtype=np.float32)[truth] + rng.normal(0, 0.08, size=truth.shape).astype(np.float32)
    data = _nll(img, means, 0.08, clamp_hi=20.0, shift_nonneg=False)
    parent = [-1, 0, 0, 0]
    return Workload("boxes64_flat3", (n, n, n), parent, {1 + k: data[k] for k in range(3)},
                    alpha={v: 0.1 for v in (1, 2, 3)}, iterations=iterations, truth=truth)


def ellipsoids_tree4(seed=0, size=256, iterations=500) -> Workload:
    """256^3, 4 seeded ellipsoids (radii U[20,80], means U(0.1,0.9), painted in
    order, background = class 0), sigma 0.05; tree root -> {B1: {L0, L1},
    B2: {L2, L3}}; D = Gaussian NLL shifted to >= 0; per-voxel smoothness
    0.2*exp(-|grad I|^2/0.01) shared by every vertex, alpha 1."""
    rng = np.random.default_rng(seed)
    shape = (size, size, size)
    truth = _ellipsoid_labels(shape, 4, rng, 20 * size / 256, 80 * size / 256)
    means = rng.uniform(0.1, 0.9, size=4)
    img = means.astype(np.float32)[truth] + rng.normal(0, 0.05, size=shape).astype(np.float32)
    data = _nll(img, means, 0.05)
    S = _grad_smoothness(img, 0.2, 0.01)
    # vertices: 0 root, 1 B1, 2 L0, 3 L1, 4 B2, 5 L2, 6 L3
    parent = [-1, 0, 1, 1, 0, 4, 4]
    leaves = [2, 3, 5, 6]
    return Workload("ellipsoids256_tree4", (size, size, size), parent,
                    {leaves[k]: data[k] for k in range(4)},
                    smooth={v: S for v in range(1, 7)}, alpha={v: 1.0 for v in range(1, 7)},
                    iterations=iterations, truth=truth)


def ellipsoids_flat4(seed=0, size=128, iterations=300) -> Workload:
    """128^3, 4 ellipsoids, sigma 0.1, flat 4 leaves, alpha 0.1 per leaf."""
    rng = np.random.default_rng(seed)
    shape = (size, size, size)
    truth = _ellipsoid_labels(shape, 4, rng, 10 * size / 128, 40 * size / 128)
    means = rng.uniform(0.1, 0.9, size=4)
    img = means.astype(np.float32)[truth] + rng.normal(0, 0.1, size=shape).astype(np.float32)
    data = _nll(img, means, 0.1)
    parent = [-1, 0, 0, 0, 0]
    return Workload("ellipsoids128_flat4", (size, size, size), parent, {1 + k: data[k] for k in range(4)},
                    alpha={v: 0.1 for v in range(1, 5)}, iterations=iterations, truth=truth)


def batch_flat3(seed=0, count=64, lo=48, hi=192, iterations=200) -> list[Workload]:
    """`count` volumes with per-axis sizes U{lo..hi}, 3-ellipsoid phantoms,
    sigma 0.08, flat 3 leaves, alpha 0.15."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        vx, vy, vz = (int(v) for v in rng.integers(lo, hi + 1, size=3))
        shape = (vz, vy, vx)
        r = min(shape) / 6
        truth = _ellipsoid_labels(shape, 3, rng, r, 2.5 * r)
        means = rng.uniform(0.1, 0.9, size=3)
        img = means.astype(np.float32)[truth] + rng.normal(0, 0.08, size=shape).astype(np.float32)
        data = _nll(img, means, 0.08)
        out.append(Workload("batch%02d" % i, (vx, vy, vz), [-1, 0, 0, 0], {1 + k: data[k] for k in range(3)},
                            alpha={v: 0.15 for v in (1, 2, 3)}, iterations=iterations, truth=truth))
    return out


def ellipsoids_tree8(seed=0, dims=(512, 512, 384), iterations=400) -> Workload:
    """512x512x384 CT-like phantom, 8 nested/overlapping ellipsoids, means
    U(0,1), sigma 0.03; tree root -> 2 -> 4 -> 8; smoothness
    0.1*exp(-|grad I|^2/0.005) shared."""
    rng = np.random.default_rng(seed)
    vx, vy, vz = dims
    shape = (vz, vy, vx)
    s = min(dims) / 384
    truth = _ellipsoid_labels(shape, 8, rng, 40 * s, 160 * s)
    means = rng.uniform(0.0, 1.0, size=8)
    img = means.astype(np.float32)[truth] + rng.normal(0, 0.03, size=shape).astype(np.float32)
    data = _nll(img, means, 0.03)
    S = _grad_smoothness(img, 0.1, 0.005)
    # 0 root; 1,2 level-1; 3..6 level-2; 7..14 leaves
    parent = [-1, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6]
    leaves = list(range(7, 15))
    return Workload("ellipsoids512x512x384_tree8", dims, parent, {leaves[k]: data[k] for k in range(8)},
                    smooth={v: S for v in range(1, 15)}, alpha={v: 1.0 for v in range(1, 15)},
                    iterations=iterations, truth=truth)


def random_tree_problem(seed, dims, parent, iterations=20, smooth_nodes=(), alpha_range=(0.05, 1.0),
                        data_hi=3.0) -> Workload:
    """Small random problem for parity tests: uniform data terms, random
    smoothness images on some vertices, random alpha."""
    rng = np.random.default_rng(seed)
    vx, vy, vz = dims
    shape = (vz, vy, vx)
    kids = {v: 0 for v in range(len(parent))}
    for p in parent:
        if p >= 0:
            kids[p] += 1
    data = {v: rng.uniform(0, data_hi, size=shape).astype(np.float32)
            for v in range(len(parent)) if kids[v] == 0 and parent[v] >= 0}
    smooth = {v: rng.uniform(0, 1, size=shape).astype(np.float32) for v in smooth_nodes}
    alpha = {v: float(rng.uniform(*alpha_range)) for v in range(len(parent)) if parent[v] >= 0}
    return Workload("random", tuple(dims), list(parent), data, smooth, alpha, iterations)
