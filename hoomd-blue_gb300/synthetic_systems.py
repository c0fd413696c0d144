"""Seeded synthetic systems for the benchmark configurations (no dataset is involved).

This module needs numpy only: it loads no compiled code, so the CPU reference timing and the
GPU path build their inputs from the same generators. Each generator returns a ``HostSystem``
(box, positions, type ids, type names, velocities) with the attribute layout of a snapshot
(``.configuration.box``, ``.particles.N/position/typeid/types/velocity``);
``hoomd_gb300.workloads`` turns them into ``hoomd_gb300.Snapshot`` objects.

* ``lj_fluid_sc``: N = n^3 particles on a simple-cubic lattice in a cubic box at a given number
  density, each position jittered uniformly by +-jitter (the 4096-particle LJ fluid: n = 16,
  density 0.84, jitter 0.05).
* ``lj_fluid_fcc``: N = 4 m^3 particles on an FCC lattice (the 1,048,576-particle LJ fluid:
  m = 64, density 0.84, jitter 0.05).
* ``binary_mixture``: N particles, 80 % A / 20 % B by seeded shuffle, on a jittered simple-cubic
  lattice at the given density (a Kob-Andersen start that needs no overlap removal).
* ``replica_systems``: independent single-type LJ systems with N ~ U[n_min, n_max], density
  ~ U[0.7, 0.9] and kT ~ U[0.8, 2.0]; particles on randomly chosen sites of the smallest simple-
  cubic lattice with at least N sites, jittered, Maxwell-Boltzmann velocities at kT with zero
  net momentum (the 256-replica ensemble: count 256, N in [500, 20000]).
* ``multitype_system`` and ``mixture_tables``: N particles of uniformly random types and the
  per-pair tabulated potentials (LJ + Yukawa + Gaussian, F = -dU/dr analytic) on HOOMD's table
  grid r_k = r_min + k (r_cut - r_min)/width.
"""

import numpy as np


class _HostConfiguration:
    def __init__(self, box):
        self.box = [float(x) for x in box]
        self.dimensions = 3


class _HostParticles:
    def __init__(self, pos, types, typeid):
        self.N = len(pos)
        self.types = list(types)
        self.position = np.asarray(pos, np.float64)
        self.typeid = np.asarray(typeid, np.uint32)
        self.velocity = np.zeros((self.N, 3), np.float64)


class HostSystem:
    """A generated system in plain numpy arrays (tag order = array order)."""

    def __init__(self, pos, L, types, typeid):
        self.configuration = _HostConfiguration([L, L, L, 0, 0, 0])
        self.particles = _HostParticles(pos, types, typeid)


def _snapshot(pos, L, types, typeid):
    return HostSystem(pos, L, types, typeid)


def sc_positions(n, a):
    """Simple-cubic lattice in the ordering of the reference's lattice_snapshot_factory
    (hoomd/conftest.py:203-253): numpy.meshgrid over arange(-n/2, n/2), offset by 0.5 a."""
    ranges = [np.arange(-n / 2, n / 2) for _ in range(3)]
    x, y, z = np.meshgrid(*ranges)
    return (np.vstack((x.flatten(), y.flatten(), z.flatten())).T + 0.5) * a


def lj_fluid_sc(n=16, density=0.84, jitter=0.05, seed=1, types=("A",)):
    N = n ** 3
    L = (N / density) ** (1.0 / 3.0)
    pos = sc_positions(n, L / n)
    rng = np.random.default_rng(seed)
    pos = pos + rng.uniform(-jitter, jitter, pos.shape)
    return _snapshot(pos, L, types, np.zeros(N, np.uint32))


def lj_fluid_fcc(m=64, density=0.84, jitter=0.05, seed=1):
    N = 4 * m ** 3
    L = (N / density) ** (1.0 / 3.0)
    a = L / m
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.arange(m)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pos = ((cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) + 0.25) * a - L / 2
    rng = np.random.default_rng(seed)
    pos = pos + rng.uniform(-jitter, jitter, pos.shape)
    return _snapshot(pos, L, ("A",), np.zeros(N, np.uint32))


def binary_mixture(N=262144, density=1.2, frac_a=0.8, jitter=0.05, seed=1):
    n = int(round(N ** (1.0 / 3.0)))
    if n ** 3 != N:
        raise ValueError("binary_mixture places particles on an n^3 lattice")
    L = (N / density) ** (1.0 / 3.0)
    pos = sc_positions(n, L / n)
    rng = np.random.default_rng(seed)
    pos = pos + rng.uniform(-jitter, jitter, pos.shape)
    typeid = np.zeros(N, np.uint32)
    typeid[int(round(frac_a * N)):] = 1
    rng.shuffle(typeid)
    return _snapshot(pos, L, ("A", "B"), typeid)


KOB_ANDERSEN = {("A", "A"): (1.0, 1.0), ("A", "B"): (1.5, 0.8), ("B", "B"): (0.5, 0.88)}


def multitype_system(N=524288, ntypes=32, density=0.8, jitter=0.05, seed=1):
    n = int(round(N ** (1.0 / 3.0)))
    if n ** 3 == N:
        L = (N / density) ** (1.0 / 3.0)
        pos = sc_positions(n, L / n)
    else:
        L = (N / density) ** (1.0 / 3.0)
        m = int(np.ceil(N ** (1.0 / 3.0)))
        pos = sc_positions(m, L / m)[:N]
    rng = np.random.default_rng(seed)
    pos = pos + rng.uniform(-jitter, jitter, pos.shape)
    typeid = rng.integers(0, ntypes, N).astype(np.uint32)
    types = [f"T{k}" for k in range(ntypes)]
    return _snapshot(pos, L, types, typeid)


def mixture_tables(ntypes=32, r_min=0.8, r_cut=3.0, width=1000, seed=2):
    """Per unordered type pair: LJ(eps~U[0.5,1.5], sigma~U[0.8,1.2]) + Yukawa(A~U[-2,2],
    kappa~U[0.5,3]) + Gaussian(A~U[0,2], w~U[0.1,0.4]) on r_k = r_min + k dr, dr =
    (r_cut - r_min)/width. Returns {(i, j): dict(r_min, U, F, coeffs)} for i <= j."""
    rng = np.random.default_rng(seed)
    r = np.linspace(r_min, r_cut, width, endpoint=False)
    out = {}
    for i in range(ntypes):
        for j in range(i, ntypes):
            eps, sig = rng.uniform(0.5, 1.5), rng.uniform(0.8, 1.2)
            A, kap = rng.uniform(-2, 2), rng.uniform(0.5, 3)
            G, w = rng.uniform(0, 2), rng.uniform(0.1, 0.4)
            c = dict(eps=eps, sig=sig, A=A, kappa=kap, G=G, w=w)
            U, F = table_potential(r, **c)
            out[(i, j)] = dict(r_min=r_min, U=U, F=F, coeffs=c)
    return out


def table_potential(r, eps, sig, A, kappa, G, w):
    sr6 = (sig / r) ** 6
    ey = np.exp(-kappa * r)
    eg = np.exp(-0.5 * (r / w) ** 2)
    U = 4 * eps * (sr6 * sr6 - sr6) + A * ey / r + G * eg
    F = 4 * eps * (12 * sr6 * sr6 - 6 * sr6) / r + A * ey * (kappa * r + 1) / (r * r) + G * eg * r / (w * w)
    return U, F


def replica_systems(count=256, n_min=500, n_max=20000, rho=(0.7, 0.9), kT=(0.8, 2.0),
                    jitter=0.05, seed=4):
    """[(snapshot, kT, seed)] for ``count`` replicas drawn from one seeded generator."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(count):
        N = int(rng.integers(n_min, n_max + 1))
        density = float(rng.uniform(*rho))
        kt = float(rng.uniform(*kT))
        L = (N / density) ** (1.0 / 3.0)
        m = int(np.ceil(N ** (1.0 / 3.0) - 1e-9))
        sites = np.sort(rng.choice(m ** 3, N, replace=False))
        pos = sc_positions(m, L / m)[sites] + rng.uniform(-jitter, jitter, (N, 3))
        vel = rng.normal(0.0, np.sqrt(kt), (N, 3))
        vel -= vel.mean(axis=0)
        s = _snapshot(pos, L, ("A",), np.zeros(N, np.uint32))
        s.particles.velocity[:] = vel
        out.append((s, kt, r + 1))
    return out
