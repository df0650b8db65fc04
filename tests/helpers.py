"""Shared problem builders for the parity tests (seeded synthetic inputs)."""
import numpy as np

MU0 = 4e-7 * np.pi


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def random_unit(n, seed):
    """Counter-based N(0,1) triples (SplitMix64 + Box-Muller in FP64), normalised."""
    idx = np.arange(6 * n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + idx * np.uint64(0x9E3779B97F4A7C15))
        z = key + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = ((z >> np.uint64(11)).astype(np.float64) + 0.5) / float(1 << 53)
    u = u.reshape(n, 6)
    r1 = np.sqrt(-2.0 * np.log(u[:, 0])); r2 = np.sqrt(-2.0 * np.log(u[:, 2]))
    g = np.stack([r1 * np.cos(2 * np.pi * u[:, 1]), r1 * np.sin(2 * np.pi * u[:, 1]),
                  r2 * np.cos(2 * np.pi * u[:, 3])], axis=1)
    return g / np.linalg.norm(g, axis=1, keepdims=True)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64); b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def problem(nx, ny, nz, d=(4e-9, 4e-9, 4e-9), ms=8e5, a_ex=1.3e-11, alpha=0.5, b_mt=(10.0, 5.0, 0.0),
            seed=0, **extra):
    n = nx * ny * nz
    kw = dict(nx=nx, ny=ny, nz=nz, dx=d[0], dy=d[1], dz=d[2], ms=ms, a_ex=a_ex, alpha=alpha,
              gamma=2.211e5, m0=random_unit(n, seed))
    if b_mt is not None:
        kw["h_ext"] = tuple(b * 1e-3 / MU0 for b in b_mt)
    kw.update(extra)
    return kw
