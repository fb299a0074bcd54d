"""Replicas over independent frames: one process per GPU, each evaluating
its own frames with no collective inside the step (the frames of a batch
share nothing), and a host-side gather of the per-frame results at the end.

The partition balances atoms, not frames: frames are taken in decreasing
size and each goes to the rank with the fewest atoms so far (ties to the
lower rank), so that ranks finish their packed steps at about the same time.
Every rank computes the same partition from the same sizes, with no
communication.
"""

from __future__ import annotations

import numpy as np


def partition_frames(natoms_per_frame, world: int) -> list[list[int]]:
    """Frame indices of every rank, each list ascending."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = np.asarray(natoms_per_frame, np.int64).reshape(-1)
    order = np.argsort(-sizes, kind="stable")
    load = np.zeros(world, np.int64)
    parts: list[list[int]] = [[] for _ in range(world)]
    for f in order:
        r = int(np.argmin(load))
        parts[r].append(int(f))
        load[r] += sizes[f]
    return [sorted(p) for p in parts]


def frames_of_rank(natoms_per_frame, world: int, rank: int) -> list[int]:
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside [0, {world})")
    return partition_frames(natoms_per_frame, world)[rank]


def gather_frame_results(frame_ids, energy, virial, forces, nframes_total: int, group=None):
    """Collect every rank's per-frame results on every rank, in the global
    frame order.  frame_ids: this rank's global frame indices; energy
    [n] and virial [n, 9] (array-likes), forces: a list of [natoms_f, 3]
    arrays, one per frame of this rank.  Returns (E [nframes_total],
    V [nframes_total, 9], F list of nframes_total arrays); raises if a frame
    is missing or claimed twice."""
    import torch.distributed as dist

    mine = {"ids": [int(f) for f in frame_ids],
            "E": np.asarray(energy, np.float64).reshape(-1),
            "V": np.asarray(virial, np.float64).reshape(-1, 9),
            "F": [np.asarray(f) for f in forces]}
    if len(mine["ids"]) != len(mine["E"]) or len(mine["ids"]) != len(mine["F"]):
        raise ValueError("frame_ids, energy and forces must have one entry per frame")
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    allp = [None] * world
    if world > 1:
        dist.all_gather_object(allp, mine, group=group)
    else:
        allp = [mine]
    E = np.full(nframes_total, np.nan)
    V = np.full((nframes_total, 9), np.nan)
    F: list = [None] * nframes_total
    for part in allp:
        for k, f in enumerate(part["ids"]):
            if F[f] is not None:
                raise RuntimeError(f"frame {f} gathered twice")
            E[f], V[f], F[f] = part["E"][k], part["V"][k], part["F"][k]
    missing = [f for f in range(nframes_total) if F[f] is None]
    if missing:
        raise RuntimeError(f"frames {missing[:8]} missing from the gather")
    return E, V, F
