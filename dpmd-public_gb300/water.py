"""Seeded synthetic water frames (the stand-in for the reference's water
training fixture ``source/tests/pt/model/water/data``: O/H types, ~1 g/cm^3,
PBC cubic boxes).

Geometry: molecules on a cubic lattice, O at the site, two H at 0.9572 A with
an H-O-H angle of 104.52 deg, each molecule rotated by a uniform random
rotation, every atom jittered by N(0, sigma^2), then wrapped into the box.
Atom order per molecule is [O, H, H]; types O = 0, H = 1.  All randomness
comes from ``numpy.random.default_rng(seed)`` (PCG64).
"""

from __future__ import annotations

import math

import numpy as np

OH = 0.9572
HOH_DEG = 104.52
# 1.0 g/cm^3 water: 0.033428 molecules / A^3  ->  29.915 A^3 per molecule
VOL_PER_MOLECULE = 29.915


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotations from uniform unit quaternions (Shoemake)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack(
        [
            np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
            np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
            np.sqrt(u1) * np.sin(2 * np.pi * u3),
            np.sqrt(u1) * np.cos(2 * np.pi * u3),
        ],
        axis=1,
    )
    x, y, z, w = q.T
    return np.stack(
        [
            np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], 1),
            np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], 1),
            np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1),
        ],
        axis=1,
    )


def _molecule_template() -> np.ndarray:
    half = math.radians(HOH_DEG) / 2
    return np.array(
        [
            [0.0, 0.0, 0.0],
            [OH * math.sin(half), OH * math.cos(half), 0.0],
            [-OH * math.sin(half), OH * math.cos(half), 0.0],
        ]
    )


def water_frame(
    n_side: int,
    box_len: float,
    seed: int,
    jitter: float = 0.05,
    n_mol: int | None = None,
) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """One frame of water on an ``n_side``^3 lattice in a cubic box.

    If ``n_mol`` is given, that many lattice sites are drawn (without
    replacement, seeded) from the ``n_side``^3 sites.
    Returns (coord [natoms, 3] float64, atype [natoms] int32, box [9] float64).
    """
    rng = np.random.default_rng(seed)
    g = np.arange(n_side) * (box_len / n_side)
    sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    if n_mol is not None and n_mol < len(sites):
        sites = sites[np.sort(rng.choice(len(sites), n_mol, replace=False))]
    nm = len(sites)
    rot = _random_rotations(rng, nm)
    mol = np.einsum("nij,aj->nai", rot, _molecule_template())
    coord = (sites[:, None, :] + mol).reshape(-1, 3)
    coord = coord + rng.normal(0.0, jitter, coord.shape)
    coord = np.mod(coord, box_len)
    atype = np.tile(np.array([0, 1, 1], np.int32), nm)
    box = np.diag([box_len] * 3).reshape(-1).astype(np.float64)
    return coord, atype, box


def water_box_for(n_mol: int) -> float:
    """Cubic box edge for ``n_mol`` molecules at 1.0 g/cm^3."""
    return (n_mol * VOL_PER_MOLECULE) ** (1.0 / 3.0)


def ragged_counts(n_frames: int, seed: int, lo: int = 8, hi: int = 512) -> np.ndarray:
    """Molecule counts ~ U[lo, hi] of the frames of ``ragged_frames``."""
    return np.random.default_rng(seed).integers(lo, hi + 1, n_frames)


def ragged_frames(n_frames: int, seed: int, lo: int = 8, hi: int = 512, which=None):
    """Independent frames with molecule counts ~ U[lo, hi], each in its own
    1.0 g/cm^3 cubic box on an n = ceil(N^(1/3)) lattice.  ``which``: build
    only these frame indices (in that order); each frame has its own seed, so
    a subset equals the same frames of the whole set."""
    counts = ragged_counts(n_frames, seed, lo, hi)
    frames = []
    for k in (range(n_frames) if which is None else which):
        n = int(counts[k])
        side = math.ceil(n ** (1.0 / 3.0) - 1e-9)
        frames.append(water_frame(side, water_box_for(n), seed * 100003 + k, n_mol=n))
    return frames


def replicated_frame(cell_side: int, cell_len: float, reps: int, seed: int,
                     jitter: float = 0.05):
    """A ``cell_side``^3-molecule cell replicated ``reps``^3 times, jittered."""
    c, t, _ = water_frame(cell_side, cell_len, seed, jitter=0.0)
    rng = np.random.default_rng(seed + 1)
    shifts = np.stack(np.meshgrid(*[np.arange(reps)] * 3, indexing="ij"), -1).reshape(-1, 3)
    coord = (shifts[:, None, :] * cell_len + c[None]).reshape(-1, 3)
    coord = coord + rng.normal(0.0, jitter, coord.shape)
    L = cell_len * reps
    coord = np.mod(coord, L)
    atype = np.tile(t, len(shifts))
    box = np.diag([L] * 3).reshape(-1).astype(np.float64)
    return coord, atype, box
