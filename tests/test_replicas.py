"""Replicas over independent frames (dpmd-public_gb300/replicas.py), on CPU:
the atom-balanced frame partition, and two gloo ranks that each evaluate
their own frames (the FP64 CPU composite stands in for the GPU step) and
gather energies, virials and forces in the global frame order, compared
with one process evaluating every frame."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp


def _small_model():
    import dataclasses
    import importlib

    import oracle as O

    mdl = importlib.import_module("dpmd_public_gb300.model")
    water = importlib.import_module("dpmd_public_gb300.water")
    cfg = dataclasses.replace(mdl.SeAConfig(), neuron=(4, 8, 16), axis_neuron=4,
                              fitting=(16, 16, 16))
    params = mdl.init_params(cfg, 11)
    ems, ats, mind = [], [], np.inf
    for c, t, b in [water.water_frame(2, 6.2, 40 + s) for s in range(2)]:
        em, emd, rij, nl = O.prod_env_mat_a_pbc(c, t, b, np.zeros((2, cfg.nnei * 4)),
                                                np.ones((2, cfg.nnei * 4)), cfg.rcut,
                                                cfg.rcut_smth, list(cfg.sel))
        ems.append(em)
        ats.append(t)
        r = np.linalg.norm(rij.reshape(-1, 3), axis=1)
        mind = min(mind, r[nl >= 0].min())
    davg, dstd = mdl.stats_from_env(ems, ats, cfg)
    tabs, infos = mdl.build_tables(params, davg, dstd, mind, cfg)
    return cfg, params, davg, dstd, tabs, infos


def _frames():
    import importlib

    water = importlib.import_module("dpmd_public_gb300.water")
    return water.ragged_frames(7, seed=12, lo=8, hi=30)


def _eval(model, frame):
    import composite

    cfg, params, davg, dstd, tabs, infos = model
    c, t, b = frame
    E, F, V, _ = composite.energy_force_virial(cfg, params, davg, dstd, c, t, b, tabs, infos)
    return E, F, V


def test_partition_balances_atoms(gb):
    import importlib

    R = importlib.import_module("dpmd_public_gb300.replicas")
    rng = np.random.default_rng(0)
    sizes = rng.integers(24, 1537, 512)
    for world in (1, 2, 3, 8):
        parts = R.partition_frames(sizes, world)
        flat = sorted(f for p in parts for f in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= sizes.max()
        assert R.frames_of_rank(sizes, world, world - 1) == parts[-1]
    with pytest.raises(ValueError):
        R.frames_of_rank(sizes, 2, 2)


def _rank_main(rank, world, port, out_path):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    from __graft_entry__ import load_package

    load_package()
    import importlib

    import torch.distributed as dist

    R = importlib.import_module("dpmd_public_gb300.replicas")
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        model = _small_model()
        frames = _frames()
        ids = R.frames_of_rank([len(f[1]) for f in frames], world, rank)
        res = [_eval(model, frames[f]) for f in ids]
        E, V, F = R.gather_frame_results(ids, [r[0] for r in res], [r[2] for r in res],
                                         [r[1] for r in res], len(frames))
        if rank == 0:
            np.savez(out_path, E=E, V=V, **{f"F{k}": f for k, f in enumerate(F)})
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_partition_and_gather(gb, tmp_path):
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "gathered.npz")
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    got = np.load(out)
    model = _small_model()
    frames = _frames()
    for k, fr in enumerate(frames):
        E, F, V = _eval(model, fr)
        assert got["E"][k] == E
        np.testing.assert_array_equal(got["V"][k], V)
        np.testing.assert_array_equal(got[f"F{k}"], F)
