"""Counter-based normal generator (host side).

splitmix64 (Vigna) + Box-Muller, the same generator the CUDA kernels use for
the Lanczos breakdown vector:  for key and index j,
    h1 = splitmix64(key * 2**32 + 2 j), h2 = splitmix64(key * 2**32 + 2 j + 1)
    u1 = ((h1 >> 11) + 1) 2**-53,  u2 = (h2 >> 11) 2**-53
    x_j = sqrt(-2 ln u1) cos(2 pi u2)
It stands in for the reference's jax.random.normal draws (Lanczos start vector
solver/usbs.py:691, sketch matrix utils/maxcut_helpers.py:302), which need JAX.
"""
import numpy as np


def _splitmix64(x):
    with np.errstate(over="ignore"):
        z = x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def hash_normal(key, n):
    j = np.arange(n, dtype=np.uint64)
    base = np.uint64((int(key) << 32) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        h1 = _splitmix64(base + np.uint64(2) * j)
        h2 = _splitmix64(base + np.uint64(2) * j + np.uint64(1))
    u1 = ((h1 >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)
    u2 = (h2 >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def hash_normal_matrix(key, n, s):
    """n x s normals; column c uses key ``key * 65536 + c``."""
    return np.stack([hash_normal(key * 65536 + c, n) for c in range(s)], axis=1)


def default_q0(n):
    q = hash_normal(0, n)
    return q / np.linalg.norm(q)
