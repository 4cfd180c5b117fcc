"""Seeded synthetic point sets for the five EMST workloads.

The reference measured on i.i.d. uniform "randomCity" sets; the workloads
below keep that distribution for the uniform case and add the clustered and
curve-like sets the throughput targets are quoted on.  All generators use
numpy's PCG64 with a fixed seed and return float32 (n, dim) arrays.

  uniform2d_1e4     2D, 10,000 points, U[0,1]^2, seed 1
  gauss3d_1e6       3D, 1,000,000 points: 90% from 64 axis-aligned anisotropic
                    Gaussians (centres U[0,1]^3, per-axis sigma log-uniform in
                    [1e-3, 1e-1], cluster chosen uniformly) + 10% U[0,1]^3,
                    clipped to the unit cube, seed 2
  bezier2d_1e7      2D, 10,000,000 points: 95% on 256 cubic Bezier curves
                    (4 control points U[0,1]^2, t ~ U[0,1], offset along the unit
                    normal by N(0, 1e-4)) + 5% U[0,1]^2, clipped, seed 3
  batch512          512 clouds, sizes floor(exp U[ln 1e3, ln 1e5]), 256 2D +
                    256 3D (seeded shuffle), each uniform or an 8-cluster Gaussian
                    (sigma 0.02, clipped) by a fair coin, seed 4
  gauss3d_1e7       3D, 10,000,000 points, the gauss3d generator with 256
                    clusters, seed 5
"""
import numpy as np


def uniform(n, dim, seed):
    return np.random.default_rng(seed).random((n, dim), dtype=np.float64).astype(np.float32)


def gauss_mixture(n, dim, n_clusters, seed, background=0.10, sigma_range=(1e-3, 1e-1)):
    rng = np.random.default_rng(seed)
    centres = rng.random((n_clusters, dim))
    lo, hi = np.log(sigma_range[0]), np.log(sigma_range[1])
    sig = np.exp(rng.uniform(lo, hi, (n_clusters, dim)))
    n_bg = int(round(n * background))
    n_cl = n - n_bg
    lab = rng.integers(0, n_clusters, n_cl)
    pts = np.empty((n, dim), np.float64)
    pts[:n_cl] = centres[lab] + rng.standard_normal((n_cl, dim)) * sig[lab]
    pts[n_cl:] = rng.random((n_bg, dim))
    perm = rng.permutation(n)
    return np.clip(pts[perm], 0.0, 1.0).astype(np.float32)


def bezier_curves(n, n_curves, seed, background=0.05, noise=1e-4):
    rng = np.random.default_rng(seed)
    ctrl = rng.random((n_curves, 4, 2))
    n_bg = int(round(n * background))
    n_c = n - n_bg
    out = np.empty((n, 2), np.float64)
    chunk = 1 << 21
    for s in range(0, n_c, chunk):
        m = min(chunk, n_c - s)
        c = rng.integers(0, n_curves, m)
        t = rng.random(m)[:, None]
        P0, P1, P2, P3 = (ctrl[c, k] for k in range(4))
        u = 1.0 - t
        pos = u ** 3 * P0 + 3 * u * u * t * P1 + 3 * u * t * t * P2 + t ** 3 * P3
        der = 3 * u * u * (P1 - P0) + 6 * u * t * (P2 - P1) + 3 * t * t * (P3 - P2)
        nrm = np.stack([-der[:, 1], der[:, 0]], 1)
        nn = np.linalg.norm(nrm, axis=1, keepdims=True)
        nn[nn == 0] = 1.0
        out[s:s + m] = pos + (nrm / nn) * rng.normal(0.0, noise, (m, 1))
    out[n_c:] = rng.random((n_bg, 2))
    perm = rng.permutation(n)
    return np.clip(out[perm], 0.0, 1.0).astype(np.float32)


def batch_clouds(n_clouds=512, seed=4, size_range=(1e3, 1e5)):
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(size_range[0]), np.log(size_range[1]), n_clouds))).astype(np.int64)
    dims = np.array([2] * (n_clouds // 2) + [3] * (n_clouds - n_clouds // 2))
    rng.shuffle(dims)
    clouds = []
    for i in range(n_clouds):
        n, d = int(sizes[i]), int(dims[i])
        if rng.random() < 0.5:
            p = rng.random((n, d))
        else:
            c = rng.random((8, d))
            p = c[rng.integers(0, 8, n)] + rng.standard_normal((n, d)) * 0.02
        clouds.append(np.clip(p, 0.0, 1.0).astype(np.float32))
    return clouds


WORKLOADS = {
    "uniform2d_1e4": lambda: uniform(10_000, 2, 1),
    "gauss3d_1e6": lambda: gauss_mixture(1_000_000, 3, 64, 2),
    "bezier2d_1e7": lambda: bezier_curves(10_000_000, 256, 3),
    "gauss3d_1e7": lambda: gauss_mixture(10_000_000, 3, 256, 5),
}


def make(name, n=None):
    """Named workload; with n, the same generator at another size (for smaller parity cases)."""
    if n is None:
        return WORKLOADS[name]()
    if name.startswith("uniform2d"):
        return uniform(n, 2, 1)
    if name == "gauss3d_1e6":
        return gauss_mixture(n, 3, 64, 2)
    if name == "gauss3d_1e7":
        return gauss_mixture(n, 3, 256, 5)
    if name == "bezier2d_1e7":
        return bezier_curves(n, 256, 3)
    raise KeyError(name)
