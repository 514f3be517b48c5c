"""Counter-based normal generator shared by the oracle and the CUDA path.

Oracle copy (test infrastructure).  The reference draws its random vectors from
``jax.random.normal(PRNGKey(key), (n,))`` (``solver/lanczos.py:110``,
``solver/usbs.py:691``, ``utils/maxcut_helpers.py:302``); that stream needs JAX,
so both implementations use this generator instead:

    h1 = splitmix64(key * 2**32 + 2*j),  h2 = splitmix64(key * 2**32 + 2*j + 1)
    u1 = ((h1 >> 11) + 1) * 2**-53      in (0, 1]
    u2 = (h2 >> 11) * 2**-53            in [0, 1)
    x_j = sqrt(-2 ln u1) * cos(2 pi u2)             (Box-Muller)

splitmix64 is Vigna's published 64-bit mixer.  The integer part is bit-exact on
every platform; the transcendental part agrees to the last few ulps.
"""
import numpy as np

_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    x = x.astype(np.uint64)
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def hash_normal(key: int, n: int) -> np.ndarray:
    """n standard normals from counter ``key`` (FP64)."""
    j = np.arange(n, dtype=np.uint64)
    base = np.uint64((int(key) << 32) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        h1 = _splitmix64(base + np.uint64(2) * j)
        h2 = _splitmix64(base + np.uint64(2) * j + np.uint64(1))
    u1 = ((h1 >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)
    u2 = (h2 >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def hash_normal_matrix(key: int, n: int, s: int) -> np.ndarray:
    """n x s normals; column c uses key ``key * 65536 + c``."""
    return np.stack([hash_normal(key * 65536 + c, n) for c in range(s)], axis=1)


def default_q0(n: int) -> np.ndarray:
    """Unit-norm Lanczos start vector (stands in for PRNGKey(0), solver/usbs.py:691-692)."""
    q = hash_normal(0, n)
    return q / np.linalg.norm(q)
