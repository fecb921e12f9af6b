"""Seeded synthetic workloads for the FEM-H1 clustering path.

All randomness comes from one counter-based generator (splitmix64 of seed, stream and index;
uniforms from the top 53 bits, normals by Box-Muller), so the same arrays can be rebuilt on any
machine and handed to both the GPU library and the CPU oracle.

Workloads (sizes and distributions of the benchmark configurations):
  signal1d_cfg0   T=1e4, K=2, levels alternating {1,2}, segment lengths U{500..2000}, noise N(0,1),
                  epssqr=10
  signal1d_cfg1   T=1e7, K=3, levels {0,1,2} in random order per segment, segment lengths
                  U[1e3, 1e5], noise N(0, 0.5^2), epssqr in {1, 10, 100, 1000}
  batched         256 signals, T log-uniform [1e3, 1e6], K U{2..5}, epssqr log-uniform [1, 1000],
                  sorted levels U[0, 4], segments U[T/50, T/5], noise sigma U[0.2, 1]
  multichannel    T=1e6, n=128 channels, K=8: centroids N(0, I_n), hidden labels a Markov chain
                  with self-transition 0.999 and uniform jumps to another state, X_t = theta_label +
                  N(0, 0.8^2 I), epssqr=50; values rounded to BF16 (the device's storage format)
The initial gamma follows the reference: uniform [0, 1) values written in the blocked order
k*T + t (GeneralVector::set_random, src/petscvector/algebra/vector/generalvector.cpp:7-28),
permuted to t*K + k by the TSSolver and projected when the SPG solve starts.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_G = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + _G
        z = (z ^ (z >> np.uint64(30))) * _C1
        z = (z ^ (z >> np.uint64(27))) * _C2
        return z ^ (z >> np.uint64(31))


def _key(seed: int, stream: int) -> np.uint64:
    k = _splitmix64(np.array([np.uint64(seed & 0xFFFFFFFFFFFFFFFF)], dtype=np.uint64))[0]
    return _splitmix64(np.array([k ^ np.uint64(stream & 0xFFFFFFFFFFFFFFFF)], dtype=np.uint64))[0]


def uniform(seed: int, stream: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles in [0, 1) for counters offset .. offset+n-1 of (seed, stream)."""
    k = _key(seed, stream)
    with np.errstate(over="ignore"):
        ctr = np.arange(offset, offset + n, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + k
    bits = _splitmix64(ctr) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """n standard normals (Box-Muller on pairs of uniforms)."""
    m = (n + 1) // 2
    u = uniform(seed, stream, 2 * m)
    u1 = 1.0 - u[0::2]  # (0, 1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.empty(2 * m)
    z[0::2] = r * np.cos(2.0 * np.pi * u2)
    z[1::2] = r * np.sin(2.0 * np.pi * u2)
    return z[:n]


def randint(seed: int, stream: int, n: int, lo: int, hi: int) -> np.ndarray:
    """n integers uniform in [lo, hi] inclusive."""
    u = uniform(seed, stream, n)
    return lo + np.minimum((u * (hi - lo + 1)).astype(np.int64), hi - lo)


@dataclass
class Signal1D:
    T: int
    K: int
    data: np.ndarray          # T, noisy signal
    clean: np.ndarray         # T, piecewise-constant truth
    labels: np.ndarray        # T, index of the true level
    levels: np.ndarray        # K, the true levels
    gamma0: np.ndarray        # K*T, uniform [0,1) in blocked order (reference set_random)
    epssqr: list = field(default_factory=list)
    name: str = ""


def _segments(seed, stream, T, lmin, lmax):
    nseg = T // max(lmin, 1) + 2
    lens = randint(seed, stream, nseg, lmin, lmax)
    ends = np.cumsum(lens)
    nseg = int(np.searchsorted(ends, T) + 1)
    lens = lens[:nseg].copy()
    lens[-1] -= int(ends[nseg - 1] - T)
    return lens


def signal1d(T, K, levels, seg_min, seg_max, sigma, seed, alternate=False, epssqr=None, name=""):
    """Piecewise-constant signal with Gaussian noise; levels per segment alternate (K=2
    style) or are drawn uniformly at random."""
    levels = np.asarray(levels, dtype=np.float64)
    lens = _segments(seed, 1, T, seg_min, seg_max)
    if alternate:
        lab_seg = np.arange(len(lens)) % K
    else:
        lab_seg = randint(seed, 2, len(lens), 0, K - 1)
    labels = np.repeat(lab_seg, lens).astype(np.int32)
    clean = levels[labels]
    data = clean + sigma * normal(seed, 3, T)
    gamma0 = uniform(seed, 4, K * T)
    return Signal1D(T=T, K=K, data=data, clean=clean, labels=labels, levels=levels,
                    gamma0=gamma0, epssqr=list(epssqr or []), name=name)


def signal1d_cfg0(seed: int = 0) -> Signal1D:
    return signal1d(10_000, 2, [1.0, 2.0], 500, 2000, 1.0, seed, alternate=True, epssqr=[10.0],
                    name="signal1d T=1e4 K=2 levels {1,2} sigma=1")


def signal1d_cfg1(seed: int = 1, T: int = 10_000_000) -> Signal1D:
    return signal1d(T, 3, [0.0, 1.0, 2.0], 1000, 100_000, 0.5, seed,
                    epssqr=[1.0, 10.0, 100.0, 1000.0],
                    name=f"signal1d T={T:.0e} K=3 levels {{0,1,2}} sigma=0.5")


def normalised_gamma(gamma0_blocked: np.ndarray, T: int, K: int) -> np.ndarray:
    """Interleaved gamma0 normalised onto the simplex per timestep (divide by the sum)."""
    g = gamma0_blocked.reshape(K, T).T.copy()
    g /= g.sum(axis=1, keepdims=True)
    return g.ravel()


@dataclass
class BatchInstance:
    T: int
    K: int
    epssqr: float
    sigma: float
    levels: np.ndarray
    data: np.ndarray
    clean: np.ndarray
    gamma0: np.ndarray


def batched_lengths(n: int = 256, seed: int = 3, tmin: int = 1000, tmax: int = 1_000_000) -> list[int]:
    """T of each signal of `batched` with the same arguments, without generating the signals."""
    u = uniform(seed, 100, 6 * n).reshape(n, 6)
    return [int(round(np.exp(np.log(tmin) + u[i, 0] * (np.log(tmax) - np.log(tmin))))) for i in range(n)]


def batched(n: int = 256, seed: int = 3, tmin: int = 1000, tmax: int = 1_000_000,
            indices=None) -> list[BatchInstance]:
    """The uneven batch: n signals with T log-uniform in [tmin, tmax], K uniform in 2..5,
    epssqr log-uniform in [1, 1000], sorted levels U[0, 4], segments U[T/50, T/5], noise
    U[0.2, 1].  `indices` selects which signals to generate (all of them, in order, by default);
    signal i is the same whichever others are generated."""
    u = uniform(seed, 100, 6 * n).reshape(n, 6)
    out = []
    for i in (range(n) if indices is None else indices):
        i = int(i)
        T = int(round(np.exp(np.log(tmin) + u[i, 0] * (np.log(tmax) - np.log(tmin)))))
        K = 2 + min(int(u[i, 1] * 4), 3)
        eps = float(np.exp(u[i, 2] * np.log(1000.0)))
        sigma = 0.2 + 0.8 * u[i, 3]
        levels = np.sort(4.0 * uniform(seed, 1000 + i, K))
        s = signal1d(T, K, levels, max(T // 50, 1), max(T // 5, 1), sigma, seed * 100003 + i)
        out.append(BatchInstance(T=T, K=K, epssqr=eps, sigma=sigma, levels=levels, data=s.data,
                                 clean=s.clean, gamma0=s.gamma0))
    return out


def bf16_round(x: np.ndarray) -> np.ndarray:
    """FP64 values rounded to the nearest BF16 value (ties to even), returned as FP64: the
    rounding the device applies to multichannel data (one rounding from FP64, no FP32 step)."""
    x = np.asarray(x, dtype=np.float64)
    f, e = np.frexp(x)  # |x| = |f| 2^e, |f| in [0.5, 1)
    ulp_exp = e - 8     # BF16 keeps 8 significant bits
    return np.ldexp(np.round(np.ldexp(x, -ulp_exp)), ulp_exp)


@dataclass
class Multichannel:
    T: int
    n: int
    K: int
    data: np.ndarray       # T*n row-major, BF16-representable values
    centroids: np.ndarray  # K*n
    labels: np.ndarray     # T
    gamma0: np.ndarray     # K*T, uniform [0,1) in blocked order
    epssqr: float = 50.0


def multichannel(T: int = 1_000_000, n: int = 128, K: int = 8, seed: int = 2, stay: float = 0.999,
                 sigma: float = 0.8, epssqr: float = 50.0) -> Multichannel:
    centroids = normal(seed, 1, K * n)
    jump = uniform(seed, 2, T) >= stay
    jump[0] = False
    step = randint(seed, 3, T, 1, K - 1) * jump
    labels = ((randint(seed, 6, 1, 0, K - 1)[0] + np.cumsum(step)) % K).astype(np.int32)
    data = centroids.reshape(K, n)[labels].ravel() + sigma * normal(seed, 4, T * n)
    return Multichannel(T=T, n=n, K=K, data=bf16_round(data), centroids=centroids, labels=labels,
                        gamma0=uniform(seed, 5, K * T), epssqr=epssqr)
