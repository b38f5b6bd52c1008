"""Seeded synthetic inputs (numpy), identical to the oracle's generator.

* scalars: a splitmix64 stream, four outputs per candidate as little-endian
  64-bit limbs, top bit cleared, accepted iff < r (uniform Fr, <= 255 bits);
  kind 1: one output per scalar (uniform 64-bit, bytes 8..31 zero);
  kind 2: kind 0 with a seeded ~10% of scalars set to zero.
* points: P_i = k_i * G with k_i = scalars(seed ^ 0xA5A5A5A5, n, kind 0),
  computed on the GPU by catmsm_p1_affines_from_scalars(_device).
* duplicates: a seeded ~5% of points replaced by copies of other points.

No public dataset is involved; every input is derived from a seed.
"""
import numpy as np

R = 0x73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001
_R_LIMBS = [(R >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(4)]
GAMMA = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(state: int, count: int) -> np.ndarray:
    """The first `count` outputs of splitmix64 seeded with `state`."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(state) + idx * GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _lt_r(c: np.ndarray) -> np.ndarray:
    """c: (m, 4) uint64 little-endian limbs -> bool (m,) value < r."""
    lt = np.zeros(c.shape[0], dtype=bool)
    eq = np.ones(c.shape[0], dtype=bool)
    for i in (3, 2, 1, 0):
        li = np.uint64(_R_LIMBS[i])
        lt |= eq & (c[:, i] < li)
        eq &= c[:, i] == li
    return lt


def scalars(seed: int, n: int, kind: int = 0) -> bytes:
    """n 32-byte little-endian scalars (see module docstring)."""
    if kind == 1:
        out = np.zeros((n, 4), dtype=np.uint64)
        out[:, 0] = splitmix64(seed, n)
        return out.tobytes()
    need = n
    m = int(n * 1.2) + 64
    while True:
        raw = splitmix64(seed, 4 * m).reshape(m, 4)
        raw[:, 3] &= np.uint64(0x7FFFFFFFFFFFFFFF)
        ok = _lt_r(raw)
        if int(ok.sum()) >= need:
            break
        m *= 2
    out = raw[ok][:n].copy()
    if kind == 2:
        sel = splitmix64(seed ^ 0x5EED5EED5EED5EED, n) % np.uint64(10) == 0
        out[sel] = 0
    return out.tobytes()


def point_scalars(seed: int, n: int) -> bytes:
    """The k_i with P_i = k_i * G for the seeded point set `seed`."""
    return scalars(seed ^ 0xA5A5A5A5, n, 0)


def duplicate_indices(seed: int, n: int):
    """(dst, src) index pairs of the seeded ~5% duplicated points, in order."""
    z = splitmix64(seed ^ 0xD0B1ED0B1ED0B1ED, 2 * n).reshape(n, 2)
    dst = np.nonzero(z[:, 0] % np.uint64(20) == 0)[0]
    src = (z[dst, 1] % np.uint64(n)).astype(np.int64)
    return dst, src


def apply_duplicates(points: bytearray, seed: int, n: int) -> bytearray:
    """Sequentially replace points[dst] = points[src] (same order as the oracle)."""
    dst, src = duplicate_indices(seed, n)
    for d, s in zip(dst.tolist(), src.tolist()):
        points[96 * d:96 * d + 96] = points[96 * s:96 * s + 96]
    return points
