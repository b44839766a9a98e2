"""Seeded synthetic inputs for the reconstruction path.

The reference reconstructs measured tomography data (HDF5 exchange files);
none is available here, so inputs are synthetic with the reference workloads'
shapes: random-ellipse phantoms, projected by the plan's own forward
projector, with optional Poisson counting noise.

Coordinates are normalised to the grid half-width g/2, so a phantom's look
does not depend on the grid size.
"""
from __future__ import annotations

import numpy as np


def ellipse_params(num_slices: int, seed: int, n_ellipses: int = 10):
    """Per slice and ellipse: (cx, cy, a, b, phi, intensity).

    Centres uniform in the disk of radius 0.8, semi-axes uniform in
    [0.05, 0.4], rotation uniform in [0, pi), intensity uniform in [0.1, 1].
    """
    rng = np.random.default_rng(seed)
    n = (num_slices, n_ellipses)
    r = 0.8 * np.sqrt(rng.uniform(0, 1, n))
    t = rng.uniform(0, 2 * np.pi, n)
    cx, cy = r * np.cos(t), r * np.sin(t)
    a = rng.uniform(0.05, 0.4, n)
    b = rng.uniform(0.05, 0.4, n)
    phi = rng.uniform(0, np.pi, n)
    inten = rng.uniform(0.1, 1.0, n)
    return np.stack([cx, cy, a, b, phi, inten], -1)


def ellipse_phantoms(g: int, num_slices: int, seed: int, n_ellipses: int = 10,
                     texture_sigma: float = 0.0) -> np.ndarray:
    """[S][g][g] float32 sums of random ellipses (+ optional Gaussian texture)."""
    prm = ellipse_params(num_slices, seed, n_ellipses)
    u = (np.arange(g, dtype=np.float64) + 0.5 - g / 2) / (g / 2)
    X, Y = np.meshgrid(u, u)  # [y][x]
    out = np.zeros((num_slices, g, g), np.float64)
    for s in range(num_slices):
        for cx, cy, a, b, phi, inten in prm[s]:
            c, sn = np.cos(phi), np.sin(phi)
            xr = (X - cx) * c + (Y - cy) * sn
            yr = -(X - cx) * sn + (Y - cy) * c
            out[s] += inten * ((xr / a) ** 2 + (yr / b) ** 2 <= 1.0)
    if texture_sigma > 0:
        rng = np.random.default_rng(seed + 7919)
        out += rng.normal(0.0, texture_sigma, out.shape)
    return out.astype(np.float32)


def ellipse_phantoms_torch(g: int, num_slices: int, seed: int, device,
                           n_ellipses: int = 10, texture_sigma: float = 0.0):
    """Same phantoms generated on a device with torch (for large grids)."""
    import torch

    prm = torch.as_tensor(ellipse_params(num_slices, seed, n_ellipses),
                          dtype=torch.float32, device=device)
    u = (torch.arange(g, device=device, dtype=torch.float32) + 0.5 - g / 2) / (g / 2)
    Y, X = torch.meshgrid(u, u, indexing="ij")
    out = torch.zeros((num_slices, g, g), dtype=torch.float32, device=device)
    for s in range(num_slices):
        for e in range(prm.shape[1]):
            cx, cy, a, b, phi, inten = prm[s, e]
            c, sn = torch.cos(phi), torch.sin(phi)
            xr = (X - cx) * c + (Y - cy) * sn
            yr = -(X - cx) * sn + (Y - cy) * c
            out[s] += inten * (((xr / a) ** 2 + (yr / b) ** 2) <= 1.0).float()
    if texture_sigma > 0:
        gen = torch.Generator(device=device)
        gen.manual_seed(seed + 7919)
        out += texture_sigma * torch.randn(out.shape, generator=gen, device=device)
    return out


def poisson_log(sim: np.ndarray, i0: float, seed: int, g: int) -> np.ndarray:
    """Counting noise on line integrals given in pixel units.

    Line integrals are scaled to the normalised field of view (pixel size
    2/g), counts ~ Poisson(I0 exp(-p)), and converted back with
    -log(max(n, 1)/I0) (zero counts clamp to one photon) in pixel units.
    """
    rng = np.random.default_rng(seed)
    s = 2.0 / g
    lam = i0 * np.exp(-np.asarray(sim, np.float64) * s)
    n = np.maximum(rng.poisson(lam), 1)
    return (-np.log(n / i0) / s).astype(np.float32)


def poisson_log_torch(sim, i0: float, seed: int, g: int):
    import torch

    gen = torch.Generator(device=sim.device)
    gen.manual_seed(seed)
    s = 2.0 / g
    lam = i0 * torch.exp(-sim.double() * s)
    n = torch.clamp(torch.poisson(lam, generator=gen), min=1.0)
    return (-torch.log(n / i0) / s).float()


def ellipsoid_params(n_ellipsoids: int, seed: int):
    """Per ellipsoid: (cx, cy, cz, a, b, c, q0, q1, q2, q3, intensity).

    The 2-D slice generator extended to 3-D: centres uniform in the ball of
    radius 0.8, semi-axes uniform in [0.05, 0.4], a uniformly random
    orientation (unit quaternion), intensity uniform in [0.1, 1]; coordinates
    normalised to the volume half-extent on every axis.
    """
    rng = np.random.default_rng(seed)
    n = n_ellipsoids
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = 0.8 * rng.uniform(0, 1, n) ** (1.0 / 3.0)
    ctr = d * r[:, None]
    ax = rng.uniform(0.05, 0.4, (n, 3))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    inten = rng.uniform(0.1, 1.0, n)
    return np.concatenate([ctr, ax, q, inten[:, None]], axis=1)


def _rotation(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def ellipsoid_volume_torch(g: int, num_slices: int, seed: int, device, first: int = 0,
                           count: int | None = None, n_ellipsoids: int = 10,
                           total_slices: int | None = None):
    """Slices [first, first + count) of a [total][g][g] random-ellipsoid
    volume (slice index = z), generated on a device."""
    import torch

    total = total_slices or num_slices
    count = num_slices if count is None else count
    prm = ellipsoid_params(n_ellipsoids, seed)
    u = (torch.arange(g, device=device, dtype=torch.float32) + 0.5 - g / 2) / (g / 2)
    Y, X = torch.meshgrid(u, u, indexing="ij")
    out = torch.zeros((count, g, g), dtype=torch.float32, device=device)
    for k in range(count):
        z = (first + k + 0.5 - total / 2) / (total / 2)
        for e in prm:
            R = _rotation(e[6:10])  # body axes as columns
            dz = z - e[2]
            if abs(dz) > e[3:6].max():
                continue
            dx, dy = X - float(e[0]), Y - float(e[1])
            acc = 0.0
            for i in range(3):
                t = dx * float(R[0, i]) + dy * float(R[1, i]) + float(dz * R[2, i])
                acc = acc + (t / float(e[3 + i])) ** 2
            out[k] += float(e[10]) * (acc <= 1.0).float()
    return out


def ellipsoid_params(n_ellipsoids: int, seed: int):
    """Per ellipsoid: (cx, cy, cz, a, b, c, q0, q1, q2, q3, intensity).

    The 2-D slice generator extended to 3-D: centres uniform in the ball of
    radius 0.8, semi-axes uniform in [0.05, 0.4], a uniformly random
    orientation (unit quaternion), intensity uniform in [0.1, 1]; coordinates
    normalised to the volume half-extent on every axis.
    """
    rng = np.random.default_rng(seed)
    n = n_ellipsoids
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = 0.8 * rng.uniform(0, 1, n) ** (1.0 / 3.0)
    ctr = d * r[:, None]
    ax = rng.uniform(0.05, 0.4, (n, 3))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    inten = rng.uniform(0.1, 1.0, n)
    return np.concatenate([ctr, ax, q, inten[:, None]], axis=1)


def _rotation(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def ellipsoid_volume_torch(g: int, num_slices: int, seed: int, device, first: int = 0,
                           count: int | None = None, n_ellipsoids: int = 10):
    """Slices [first, first + count) of a [num_slices][g][g] random-ellipsoid
    volume (slice index = z), generated on a device."""
    import torch

    total = num_slices
    count = num_slices - first if count is None else count
    prm = ellipsoid_params(n_ellipsoids, seed)
    u = (torch.arange(g, device=device, dtype=torch.float32) + 0.5 - g / 2) / (g / 2)
    Y, X = torch.meshgrid(u, u, indexing="ij")
    out = torch.zeros((count, g, g), dtype=torch.float32, device=device)
    for k in range(count):
        z = (first + k + 0.5 - total / 2) / (total / 2)
        for e in prm:
            R = _rotation(e[6:10])  # body axes as columns
            dz = z - e[2]
            if abs(dz) > e[3:6].max():
                continue
            dx, dy = X - float(e[0]), Y - float(e[1])
            acc = 0.0
            for i in range(3):
                t = dx * float(R[0, i]) + dy * float(R[1, i]) + float(dz * R[2, i])
                acc = acc + (t / float(e[3 + i])) ** 2
            out[k] += float(e[10]) * (acc <= 1.0).float()
    return out
