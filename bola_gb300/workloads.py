"""Seeded synthetic inputs for tests and benchmarks.

The generator is the project's own (BOLA's benches draw from the `rand`
crate's ChaCha12 StdRng, which is not reproduced): SplitMix64 over the
element counter, top 53 bits scaled to [0, 1).  Matrices are filled in
column-major element order, so a given (seed, stream, offset) always names
the same numbers whatever the shape.
"""
import zlib

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def stream_seed(seed, stream=None):
    """Independent sub-stream of `seed` named by a string (e.g. "trsm-rhs")."""
    if stream is None:
        return int(seed) & 0xFFFFFFFFFFFFFFFF
    key = np.array([(int(seed) ^ (zlib.crc32(stream.encode()) << 32)) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64)
    with np.errstate(over="ignore"):
        return int(_mix(key + _GOLDEN)[0])


def uniform01(seed, count, offset=0, stream=None):
    """count doubles uniform in [0, 1), elements offset..offset+count-1."""
    s = np.uint64(stream_seed(seed, stream))
    out = np.empty(count, dtype=np.float64)
    step = 1 << 22
    with np.errstate(over="ignore"):
        for lo in range(0, count, step):
            hi = min(count, lo + step)
            i = np.arange(offset + lo + 1, offset + hi + 1, dtype=np.uint64)
            z = _mix(s + i * _GOLDEN)
            out[lo:hi] = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return out


def uniform_matrix(m, n, seed, lo=0.0, hi=1.0, stream=None, offset=0):
    u = uniform01(seed, m * n, offset=offset, stream=stream)
    if lo != 0.0 or hi != 1.0:
        u = lo + (hi - lo) * u
    return np.asfortranarray(u.reshape((m, n), order="F"))


def gaussian_matrix(m, n, seed, stream=None):
    """Box-Muller on pairs of the uniform stream."""
    cnt = m * n
    u = uniform01(seed, 2 * ((cnt + 1) // 2), stream=stream)
    u1 = 1.0 - u[0::2]  # (0, 1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    g = np.empty(2 * u1.size)
    g[0::2] = r * np.cos(2 * np.pi * u2)
    g[1::2] = r * np.sin(2 * np.pi * u2)
    return np.asfortranarray(g[:cnt].reshape((m, n), order="F"))


def spd_matrix(n, seed, stream=None):
    """A = B B^T / n + I with B uniform [-1, 1)."""
    B = uniform_matrix(n, n, seed, -1.0, 1.0, stream=stream)
    return np.asfortranarray(B @ B.T / n + np.eye(n))


def gemm_inputs(m, n, k, seed=0):
    """DGEMM operands drawn from one stream in the order A, B, C (uniform [0,1))."""
    A = uniform_matrix(m, k, seed)
    B = uniform_matrix(k, n, seed, offset=m * k)
    C = uniform_matrix(m, n, seed, offset=m * k + k * n)
    return A, B, C
