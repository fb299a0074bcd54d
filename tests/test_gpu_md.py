"""Velocity-Verlet NVE on the fused step: the graph-captured step replays
the eager integration, and total energy is conserved over a short run
(FP64, 192 atoms, dt 0.25 fs, 40 steps: |E(t) - E(0)| / N <= 1e-5 eV).
With random weights the potential has no short-range repulsion, so longer
runs let atoms approach until the tables are clamped; the short window
checks the integrator and the force/energy consistency only."""

import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_nve_graph_matches_eager_and_conserves_energy(gb):
    gb.load_library()
    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")
    water = importlib.import_module("dpmd_public_gb300.water")
    md = importlib.import_module("dpmd_public_gb300.md")
    cfg = mdl.SeAConfig()
    stat = [water.water_frame(4, 12.42, 3000 + s) for s in range(4)]
    m = se_a.build_model(cfg, 23, stat, DEV, torch.float64)
    c, t, b = water.water_frame(4, 12.42, 77)
    v = md.maxwell_boltzmann(t, 330.0, 5)
    eager = md.NVE(m, m.batch([t], b[None]), c, v, t, dt=0.25)
    for _ in range(5):
        eager._step()
    xe = eager.x.clone()
    g = md.NVE(m, m.batch([t], b[None]), c, v, t, dt=0.25)
    g.capture()
    g.run(5)
    torch.cuda.synchronize()
    torch.testing.assert_close(g.x, xe, atol=1e-10, rtol=1e-10)
    e0 = g.total_energy()
    worst = 0.0
    for _ in range(8):
        g.run(5)
        worst = max(worst, abs(g.total_energy() - e0) / len(t))
    assert worst <= 1e-5, worst
    assert g.batch.status() == 0


def test_nve_deterministic_trajectories_are_bitwise_equal(gb):
    """Two graph-captured NVE runs from the same state in the deterministic
    mode (fixed-point force and energy sums) give the same bits after 20
    steps (FP32 model, 192 atoms)."""
    gb.load_library()
    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")
    water = importlib.import_module("dpmd_public_gb300.water")
    md = importlib.import_module("dpmd_public_gb300.md")
    cfg = mdl.SeAConfig()
    stat = [water.water_frame(4, 12.42, 3000 + s) for s in range(4)]
    m64 = se_a.build_model(cfg, 23, stat, DEV, torch.float64)
    m = se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), DEV,
                      torch.float32, m64.tables_np, m64.infos_np)
    c, t, b = water.water_frame(4, 12.42, 78)
    v = md.maxwell_boltzmann(t, 330.0, 6)
    out = []
    for _ in range(2):
        nve = md.NVE(m, m.batch([t], b[None]), c, v, t, dt=0.5, deterministic=True)
        nve.capture()
        nve.run(20)
        torch.cuda.synchronize()
        out.append((nve.x.clone(), nve.v.clone(), float(nve.E.sum())))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
