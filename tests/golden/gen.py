"""Seeded inputs of the golden cases, made with integer and basic IEEE
arithmetic only (SplitMix64 words -> 53-bit uniforms -> rational transforms),
so that numpy on any machine regenerates them bit for bit and the fixture file
needs to hold only the outputs."""
from __future__ import annotations

import numpy as np

_M64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed: int):
        self.s = seed & _M64

    def words(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            idx = np.arange(1, n + 1, dtype=np.uint64)
            z = np.uint64(self.s) + idx * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        self.s = (self.s + n * 0x9E3779B97F4A7C15) & _M64
        return z

    def uniform(self, n: int) -> np.ndarray:
        """Doubles in [0, 1) with 53 random bits."""
        return (self.words(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def integers(self, lo: int, hi: int, n: int) -> np.ndarray:
        return (lo + (self.words(n) % np.uint64(hi - lo))).astype(np.int64)

    def bell(self, n: int) -> np.ndarray:
        """A bell-shaped variate: the centred sum of four uniforms, times 1.7."""
        u = self.uniform(4 * n).reshape(4, n)
        return (u[0] + u[1] + u[2] + u[3] - 2.0) * 1.7

    def heavy(self, n: int) -> np.ndarray:
        """Positive and right-skewed: u / (1 - v) with v kept below 1."""
        u, v = self.uniform(n), self.uniform(n)
        return (u + 0.01) / (1.0 - 0.98 * v)

    def zipfish(self, n: int, k: int) -> np.ndarray:
        """Keys in [0, k) with a skewed (about 1/r) distribution."""
        u = self.uniform(n)
        return np.minimum((k * u * u * u).astype(np.int64), k - 1).astype(np.uint32)


def tile_cases():
    """Sorted single tiles: (scale, compression, weight kind, x, w)."""
    g = SplitMix64(0x7113)
    cases = []
    sizes = [1, 2, 3, 31, 33, 100, 128, 129, 300, 513, 777, 1023, 1024]
    kinds = ["int", "frac", "decay", "prior"]
    i = 0
    for n in sizes:
        for kind in kinds:
            x = np.sort(g.bell(n) * float(10 ** (i % 4 - 1)))
            if kind == "int":
                w = g.integers(1, 60, n).astype(np.float64)
            elif kind == "frac":
                w = g.uniform(n) * 5.0 + 0.01
            elif kind == "decay":
                w = np.full(n, 1.0 + float(g.uniform(1)[0]) * 2.0 ** float(g.integers(1, 60, 1)[0]))
            else:
                w = np.full(n, 3.75)
                k = int(g.integers(0, n, 1)[0]) if n > 1 else 0
                w[:k] = g.uniform(k) * 1e3 + 1e-3
                x = np.sort(np.floor(x * 4.0) / 4.0)
            cases.append((i % 4, (50.0, 100.0, 200.0)[i % 3], kind, x, w))
            i += 1
    return cases


# decayed single digests (count clock): (scale, compression, lambda, batches, batch size)
DECAY_DIGESTS = [
    (2, 200.0, 3.4657359027997265e-05, 5, 6000),   # ln2 / 20000
    (1, 100.0, 1.3862943611198906e-04, 4, 5000),   # ln2 / 5000
    (3, 100.0, 2.3104906018664842e-04, 4, 4000),   # ln2 / 3000
    (0, 100.0, 1.7328679513998633e-04, 3, 4000),   # ln2 / 4000
]


def decay_digest_batches(case: int):
    scale, comp, lam, nb, bsz = DECAY_DIGESTS[case]
    g = SplitMix64(0xD0 + case)
    return [g.heavy(bsz) * (1.0 + 0.5 * b) for b in range(nb)]


GROUPED_TIME = (2, 100.0, 0.011552453009332421, 24)  # K2, d100, ln2 / 60 s, keys


def grouped_time_batches():
    g = SplitMix64(0x71E)
    out, t = [], 0.0
    for b in range(5):
        n = int(g.integers(1500, 4000, 1)[0])
        t += 5.0 + 30.0 * float(g.uniform(1)[0])
        out.append((g.zipfish(n, GROUPED_TIME[3]), g.heavy(n) * 3.0, t))
    return out


GROUPED_K3 = (3, 100.0, 0.0, 32)


def grouped_k3_batches():
    g = SplitMix64(0x3C3)
    mu = (g.uniform(GROUPED_K3[3]) - 0.5) * 200.0
    out = []
    for b in range(3):
        n = 8000
        z = g.zipfish(n, GROUPED_K3[3])
        tail = g.uniform(n) < 0.05
        v = mu[z] + np.where(tail, g.heavy(n) * 4.0, g.bell(n))
        out.append((z, v))
    return out


QS = np.array([1e-6, 1e-4, 0.001, 0.01, 0.1, 0.25, 0.5, 0.75, 0.9, 0.99, 0.999, 1 - 1e-4, 1 - 1e-6])
