"""Seeded synthetic inputs (host-side generators of libnaivegpu, splitmix64).

The reference draws its inputs with Distributions.Uniform and an unseeded RNG
(src/MDInput.jl:175-190, assets/positions/GeneratePositions.jl); these are the
seeded equivalents with the same shapes and distributions.  Seeds 0x4E440001 ..
0x4E440005 name the five benchmark workloads.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import ptr

SEED_PLAIN_LJ = 0x4E440001
SEED_LJ_COULOMB = 0x4E440002
SEED_NS_STRESS = 0x4E440003
SEED_ENSEMBLE = 0x4E440004
SEED_ADJOINT = 0x4E440005


def _check(st, what):
    if st != 0:
        _lib.raise_for(st, None, what)


def uniform_positions(seed: int, n: int, side: float, lo: float = 0.0) -> np.ndarray:
    """Float32 positions uniform in [lo, lo + side)^3 (N x 3)."""
    out = np.empty((n, 3), np.float32)
    _check(_lib.lib().nd_synth_uniform(seed, n, lo, side, ptr(out)), "nd_synth_uniform")
    return out


def uniform_positions_mindist(seed: int, n: int, side: float, dmin: float) -> np.ndarray:
    """FP64 positions uniform in [0, side)^3, no pair closer than dmin (N x 3)."""
    out = np.empty((n, 3), np.float64)
    _check(_lib.lib().nd_synth_uniform_mindist(seed, n, side, dmin, ptr(out)),
           "nd_synth_uniform_mindist")
    return out


def cluster_positions(seed: int, n: int, nclusters: int, side: float, smin: float,
                      smax: float) -> np.ndarray:
    out = np.empty((n, 3), np.float32)
    _check(_lib.lib().nd_synth_clusters(seed, n, nclusters, side, smin, smax, ptr(out)),
           "nd_synth_clusters")
    return out


def normal(seed: int, shape, s: float = 1.0) -> np.ndarray:
    out = np.empty(shape, np.float64)
    _check(_lib.lib().nd_synth_normal(seed, out.size, s, ptr(out)), "nd_synth_normal")
    return out


def charges_pm1(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    _check(_lib.lib().nd_synth_charges(seed, n, ptr(out)), "nd_synth_charges")
    return out


def lj_system(seed: int, n: int, side: float, dmin: float = 0.8, charges: bool = False):
    """(x, v, q) of an LJ box: positions with minimum separation dmin (the
    reference collector's `minimumdistance`, MDInput.jl:260-283), velocities
    N(0,1) per component, optional +/-1 charges (half each)."""
    x = uniform_positions_mindist(seed, n, side, dmin)
    v = normal(seed ^ 0x5EED0001, (n, 3), 1.0)
    q = charges_pm1(seed ^ 0x5EED0002, n) if charges else None
    return x, v, q


def ensemble(seed: int = SEED_ENSEMBLE, nsys: int = 512, nmin: int = 256, nmax: int = 16384,
             rho=(0.6, 0.9), sigma=(0.9, 1.1), eps=(0.8, 1.2), dmin_sigma: float = 0.8):
    """Batched LJ ensemble: N_s = 4 round(exp(U[ln nmin, ln nmax]) / 4) atoms,
    density rho_s ~ U[rho], cube side L_s = (N_s / rho_s)^(1/3) with walls
    [0, L_s]^3, sigma_s ~ U[sigma], eps_s ~ U[eps]; positions with minimum
    separation dmin_sigma * sigma_s, velocities N(0, 1).  Returns a dict with
    the per-system arrays and the concatenated x, v."""
    g = np.random.default_rng(seed)
    n = (4 * np.round(np.exp(g.uniform(np.log(nmin), np.log(nmax), nsys)) / 4)).astype(np.int64)
    n = np.clip(n, 4 * ((nmin + 3) // 4), nmax)
    r = g.uniform(rho[0], rho[1], nsys)
    side = (n / r) ** (1.0 / 3.0)
    sg = g.uniform(sigma[0], sigma[1], nsys)
    ep = g.uniform(eps[0], eps[1], nsys)
    xs, vs = [], []
    for k in range(nsys):
        sk = (seed * 1000003 + k) & 0xFFFFFFFFFFFFFFFF
        xs.append(uniform_positions_mindist(sk, int(n[k]), float(side[k]), dmin_sigma * sg[k]))
        vs.append(normal(sk ^ 0x5EED0001, (int(n[k]), 3), 1.0))
    lo = np.zeros((nsys, 3))
    hi = np.repeat(side[:, None], 3, axis=1)
    return dict(n_atoms=n, rho=r, side=side, sigma=sg, epsilon=ep, box_lo=lo, box_hi=hi,
                x=np.concatenate(xs), v=np.concatenate(vs))
