"""Seeded synthetic candidate sets with the shapes of the benchmark configurations.

The reference measures on no public dataset; every workload is synthetic:
  single     n = 32768, k odd uniform in [3, 9999]              (seed 1)
  large      n = 1,048,576, k odd uniform in [3, 2^20), x0 = a   (seed 2)
  uniform    4096 candidates, n = 65536, k odd in [3, 10^6)     (seed 3)
  uneven     2048 candidates, n log-uniform in [8192, 262144],
             k odd in [3, 10^5)                                 (seed 4)
  serving    Poisson arrivals, n log-uniform in [10000, 300000],
             k odd in [3, 10^5), trial-division pre-filter      (seed 5)
"""
import math

import numpy as np


def odd_k(rng, hi, size=None):
    """k = 2u + 1 uniform over the odd integers in [3, hi)."""
    return 2 * rng.integers(1, (hi - 2) // 2 + 1, size=size) + 1


def single(count=1, seed=1):
    rng = np.random.default_rng(seed)
    ks = odd_k(rng, 10000, size=count)
    return [(int(k), 32768) for k in ks]


def large(seed=2):
    rng = np.random.default_rng(seed)
    return int(odd_k(rng, 1 << 20)), 1 << 20


def uniform(count=4096, seed=3):
    rng = np.random.default_rng(seed)
    ks = odd_k(rng, 10 ** 6, size=count)
    return [(int(k), 65536) for k in ks]


def uneven(count=2048, seed=4):
    rng = np.random.default_rng(seed)
    ns = np.floor(np.exp(rng.uniform(math.log(8192), math.log(262144), size=count))).astype(np.int64)
    ks = odd_k(rng, 10 ** 5, size=count)
    return [(int(k), int(n)) for k, n in zip(ks, ns)]


def serving(count, rate, seed=5):
    """(arrival_time_s, k, n) with exponential inter-arrival times at `rate` per second."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    ts = np.cumsum(gaps)
    ns = np.floor(np.exp(rng.uniform(math.log(10000), math.log(300000), size=count))).astype(np.int64)
    ks = odd_k(rng, 10 ** 5, size=count)
    return [(float(t), int(k), int(n)) for t, k, n in zip(ts, ks, ns)]
