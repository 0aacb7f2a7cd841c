"""Seeded synthetic frames in the reference's simple-cubic site order.

``sc_sites`` follows AtomDistribution's "sc" distribution
(src/tools/AtomDistribution.cpp:205-240): integer sites (i, j, k) with i
fastest, then j, then k.  The workloads below add i.i.d. Gaussian jitter from
``numpy.random.default_rng(seed)``.  They stand in for the trajectories the
reference's benchmarks would read; every size and distribution is the one the
workload names.
"""
from __future__ import annotations

import math

import numpy as np


def sc_sites(n: int) -> np.ndarray:
    """First n sites of the smallest m^3 cube, x fastest (integer coordinates)."""
    m = int(math.ceil(round(n ** (1.0 / 3.0), 9)))
    while m ** 3 < n:
        m += 1
    k, j, i = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    return np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)[:n].astype(np.float64)


def jittered_lattice(n: int, spacing: float, sigma: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return sc_sites(n) * spacing + rng.normal(0.0, sigma, size=(n, 3))


def cubic_box(L: float) -> np.ndarray:
    return np.diag([L, L, L]).astype(np.float64)


# --- the five benchmark workloads ----------------------------------------

def workload_c0(frame: int = 0, seed: int = 2024):
    """1,000 atoms, 10^3 lattice at 0.30 nm, sigma 0.03, box 3.0 nm; each frame re-jittered."""
    rng = np.random.default_rng([seed, frame])
    pos = sc_sites(1000) * 0.30 + rng.normal(0.0, 0.03, size=(1000, 3))
    return pos, cubic_box(3.0)


def workload_c1(n_frames: int = 1, seed: int = 2025, step_sigma: float = 0.002):
    """32,768 atoms, 32^3 lattice at 0.31 nm, sigma 0.03, box 9.92 nm; frames are Gaussian steps."""
    rng = np.random.default_rng(seed)
    pos = sc_sites(32768) * 0.31 + rng.normal(0.0, 0.03, size=(32768, 3))
    frames = [pos]
    for _ in range(n_frames - 1):
        frames.append(frames[-1] + rng.normal(0.0, step_sigma, size=pos.shape))
    return np.stack(frames), cubic_box(9.92)


def workload_c2_system(seed: int = 2026):
    """100,000 atoms: first sites of a 47^3 lattice at 0.31 nm, sigma 0.03, box 14.5 nm."""
    rng = np.random.default_rng(seed)
    pos = sc_sites(100000) * 0.31 + rng.normal(0.0, 0.03, size=(100000, 3))
    return pos, cubic_box(14.5)


def workload_c2_actions(n_actions: int = 256, n_atoms: int = 100000, seed: int = 2027):
    """Contiguous GROUPA ranges with log-uniform sizes in [16, 4096] and R_0 ~ U(0.25, 0.45)."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(16), np.log(4096), n_actions))).astype(np.int64)
    starts = np.array([rng.integers(0, n_atoms - s + 1) for s in sizes], dtype=np.int64)
    r0 = rng.uniform(0.25, 0.45, n_actions)
    return sizes, starts, r0


def workload_c4_walker(walker: int, seed: int = 2028):
    """262,144 atoms, 64^3 lattice at 19.87/64 nm, sigma 0.03, box 19.87 nm; one seed per walker."""
    rng = np.random.default_rng([seed, walker])
    a = 19.87 / 64.0
    pos = sc_sites(262144) * a + rng.normal(0.0, 0.03, size=(262144, 3))
    return pos, cubic_box(19.87)
