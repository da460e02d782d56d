"""Seeded synthetic systems and random-init weights for the benchmark workloads.

No public dataset is involved: every input is generated from a seed with
``numpy.random.default_rng``. Shapes, sizes and value distributions follow the
workload descriptions:

* water: O on a cubic lattice (3.1 A, or box/16 for the periodic box) with
  U(-0.2, 0.2) A jitter per coordinate; each H at 0.96 A from its O with an
  H-O-H angle of 104.5 degrees, in a uniformly random orientation per molecule;
* CHNO molecules: 8-64 atoms, elements H/C/N/O with probabilities
  0.5/0.3/0.1/0.1, placed by a random-walk tree with bond lengths U(1.0, 1.5) A,
  rejecting any atom closer than 0.9 A to another;
* weights: truncated normal (re-drawn beyond 2 sigma, like TF's
  ``truncated_normal`` used by ``Instance._variable_with_weight_decay``,
  TFNetworks/TFInstance.py:277-297) with sigma = 1/(10 + sqrt(fan_in)) and zero
  biases (TFBehlerParinelloSymEE.py:917-927, 978-992);
* velocities: Maxwell-Boltzmann at T with the centre-of-mass momentum removed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .params import ATOMICMASSES, IDEALGASR


@dataclass
class System:
    """A batch of molecules in CSR layout (atoms of molecule m are
    ``offsets[m]:offsets[m+1]``)."""
    x: np.ndarray                 # [N, 3] float64, Angstrom
    Z: np.ndarray                 # [N] int32 atomic numbers
    offsets: np.ndarray           # [nmol + 1] int64
    cell: np.ndarray | None = None  # [3, 3] lattice vectors (rows) or None
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def natoms(self) -> int:
        return int(self.x.shape[0])

    @property
    def nmol(self) -> int:
        return int(self.offsets.shape[0] - 1)

    def molecule(self, m):
        a, b = int(self.offsets[m]), int(self.offsets[m + 1])
        return self.x[a:b], self.Z[a:b]


def _random_frames(rng, n):
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    w = np.cross(u, rng.normal(size=(n, 3)))
    w /= np.linalg.norm(w, axis=1)[:, None]
    return u, w


def water_sites(n_side, nmol, spacing):
    idx = np.array([[i, j, k] for i in range(n_side) for j in range(n_side)
                    for k in range(n_side)], dtype=np.float64)[:nmol]
    return idx * spacing


def water(nmol, seed, spacing=3.1, box=None, n_side=None):
    """nmol water molecules on a jittered cubic lattice; O,H,H per molecule."""
    rng = np.random.default_rng(seed)
    if n_side is None:
        n_side = int(math.ceil(round(nmol ** (1.0 / 3.0), 9)))
        while n_side ** 3 < nmol:
            n_side += 1
    O = water_sites(n_side, nmol, spacing) + rng.uniform(-0.2, 0.2, (nmol, 3))
    u, w = _random_frames(rng, nmol)
    half = math.radians(104.5) / 2.0
    H1 = O + 0.96 * (math.cos(half) * u + math.sin(half) * w)
    H2 = O + 0.96 * (math.cos(half) * u - math.sin(half) * w)
    x = np.stack([O, H1, H2], 1).reshape(-1, 3)
    cell = None
    if box is not None:
        x = np.mod(x, box)
        cell = np.eye(3) * box
    Z = np.tile(np.array([8, 1, 1], dtype=np.int32), nmol)
    return System(x=np.ascontiguousarray(x), Z=Z,
                  offsets=np.array([0, x.shape[0]], dtype=np.int64), cell=cell,
                  name=f"water{nmol}" + ("_pbc" if box is not None else ""))


def water_cluster_60(seed=0):
    """20 H2O open cluster (60 atoms)."""
    return water(20, seed, 3.1)


def water_cube_24k(seed=1):
    """8,000 H2O open-boundary cube (24,000 atoms)."""
    return water(8000, seed, 3.1)


def water_box_12k(seed=2):
    """4,096 H2O periodic box, cubic cell of side 49.7 A (12,288 atoms)."""
    return water(4096, seed, 49.7 / 16.0, box=49.7, n_side=16)


_CHNO = np.array([1, 6, 7, 8], dtype=np.int32)
_CHNO_P = np.array([0.5, 0.3, 0.1, 0.1])


def chno_molecule(rng, natoms):
    """One random-walk-tree CHNO molecule."""
    Z = rng.choice(_CHNO, size=natoms, p=_CHNO_P).astype(np.int32)
    x = np.zeros((natoms, 3))
    for a in range(1, natoms):
        for _ in range(1000):
            parent = rng.integers(0, a)
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            p = x[parent] + rng.uniform(1.0, 1.5) * d
            if np.min(np.linalg.norm(x[:a] - p, axis=1)) >= 0.9:
                x[a] = p
                break
        else:  # pragma: no cover - practically unreachable
            raise RuntimeError("random-walk placement failed")
    return x, Z


def chno_batch(nmol=512, seed=3, nmin=8, nmax=64):
    """Ragged batch of CHNO molecules with N ~ U{nmin..nmax}."""
    rng = np.random.default_rng(seed)
    xs, Zs, offs = [], [], [0]
    for _ in range(nmol):
        n = int(rng.integers(nmin, nmax + 1))
        x, Z = chno_molecule(rng, n)
        xs.append(x)
        Zs.append(Z)
        offs.append(offs[-1] + n)
    return System(x=np.ascontiguousarray(np.concatenate(xs)), Z=np.concatenate(Zs),
                  offsets=np.array(offs, dtype=np.int64), name=f"chno{nmol}")


def concat(systems):
    """Concatenate open-boundary systems into one ragged batch."""
    xs = [s.x for s in systems]
    Zs = [s.Z for s in systems]
    offs = [0]
    for s in systems:
        for m in range(s.nmol):
            offs.append(offs[-1] + int(s.offsets[m + 1] - s.offsets[m]))
    return System(x=np.ascontiguousarray(np.concatenate(xs)), Z=np.concatenate(Zs),
                  offsets=np.array(offs, dtype=np.int64), name="batch")


def truncated_normal(rng, shape, std):
    out = rng.normal(size=shape)
    bad = np.abs(out) > 2.0
    while np.any(bad):
        out[bad] = rng.normal(size=int(bad.sum()))
        bad = np.abs(out) > 2.0
    return out * std


def random_weights(eles, D, hidden=(512, 512, 512), seed=7):
    """Random-init per-element energy and charge networks.

    Returns ``{"E": {ele: [(W, b), ...]}, "Q": {...}}`` with W of shape
    [fan_in, fan_out] (the reference's ``tf.matmul(inputs, weights)``
    orientation) and one final [hidden[-1], 1] regression layer.
    """
    rng = np.random.default_rng(seed)
    out = {}
    for net in ("E", "Q"):
        out[net] = {}
        for e in eles:
            layers = []
            fan_in = D
            for h in list(hidden) + [1]:
                W = truncated_normal(rng, (fan_in, h), 1.0 / (10.0 + math.sqrt(float(fan_in))))
                b = np.zeros(h)
                layers.append((W, b))
                fan_in = h
            out[net][e] = layers
    return out


def masses(Z):
    return np.array([ATOMICMASSES[int(z)] for z in Z], dtype=np.float64)


def maxwell_boltzmann(Z, T, seed, offsets=None):
    """Velocities in A/fs at temperature T (masses in kg/mol), COM momentum
    removed per molecule."""
    rng = np.random.default_rng(seed)
    m = masses(Z)
    # <v^2> per component = R T / m in m^2/s^2; 1 m/s = 1e-5 A/fs
    sig = np.sqrt(IDEALGASR * T / m) * 1e-5
    v = rng.normal(size=(len(Z), 3)) * sig[:, None]
    if offsets is None:
        offsets = np.array([0, len(Z)])
    for a, b in zip(offsets[:-1], offsets[1:]):
        p = (m[a:b, None] * v[a:b]).sum(0) / m[a:b].sum()
        v[a:b] -= p
    return v
