"""Small seeded point families for parity tests (edge cases the reference's
uniform fixtures do not reach: clusters, ties on a lattice, exact duplicates,
collinear points)."""
import numpy as np


def family(kind, n, dim, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        return rng.random((n, dim)).astype(np.float32)
    if kind == "cluster":
        k = 8
        c = rng.random((k, dim))
        s = 10 ** rng.uniform(-3, -1, (k, dim))
        lab = rng.integers(0, k, n)
        p = c[lab] + rng.normal(size=(n, dim)) * s[lab]
        m = rng.random(n) < 0.1
        p[m] = rng.random((int(m.sum()), dim))
        return np.clip(p, 0, 1).astype(np.float32)
    if kind == "lattice":
        g = int(np.ceil(n ** (1.0 / dim)))
        pts = np.stack(np.meshgrid(*[np.arange(g)] * dim), -1).reshape(-1, dim)
        return pts[rng.permutation(len(pts))[:n]].astype(np.float32)
    if kind == "dups":
        base = rng.random((max(n // 3, 1), dim)).astype(np.float32)
        return base[rng.integers(0, len(base), n)]
    if kind == "line":
        t = np.sort(rng.random(n))
        p = np.zeros((n, dim))
        p[:, 0] = t
        p[:, 1] = t * 0.5
        return p.astype(np.float32)
    raise KeyError(kind)


KINDS = ["uniform", "cluster", "lattice", "dups", "line"]
