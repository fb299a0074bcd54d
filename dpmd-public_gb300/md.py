"""Velocity-Verlet NVE molecular dynamics on the fused se_e2_a step, with
the whole MD step (half kick, drift, energy/force/virial, half kick)
captured in a CUDA graph.

Units: eV, A, fs, amu.  The reference's MD engine is LAMMPS (out of scope);
this driver exercises the hot path the way a production MD loop does.  With
a batch made without a skin the neighbour list is rebuilt from scratch at
every step.  With a skin (Batch(skin=...)), as LAMMPS runs the reference,
every ``rebuild_every``-th step rebuilds the ghosts and an rcut + skin
Verlet list, and the steps between reuse it (the ghosts follow their atoms);
two graphs are captured, one per kind of step.  The atoms must not move by
more than half the skin between rebuilds.
"""

from __future__ import annotations

import math

import numpy as np
import torch

# 1 eV / (A amu) in A / fs^2; 1 amu A^2 / fs^2 in eV
ACC_UNIT = 9.648533212e-3
KE_UNIT = 103.6426965
KB_EV = 8.617333262e-5
MASS = {0: 15.9994, 1: 1.00794}  # O, H


def maxwell_boltzmann(atype: np.ndarray, temp: float, seed: int) -> np.ndarray:
    """Velocities (A/fs) at temperature ``temp`` (K), zero total momentum."""
    rng = np.random.default_rng(seed)
    m = np.array([MASS[int(t)] for t in atype])
    sig = np.sqrt(KB_EV * temp / (m * KE_UNIT))
    v = rng.normal(0.0, 1.0, (len(atype), 3)) * sig[:, None]
    v -= (m[:, None] * v).sum(0) / m.sum()
    return v


class NVE:
    """Graph-captured velocity-Verlet integrator for one packed batch."""

    def __init__(self, model, batch, coord: np.ndarray, vel: np.ndarray, atype: np.ndarray,
                 dt: float = 0.5, deterministic: bool | None = None, rebuild_every: int = 10):
        """deterministic: forces and energies summed in fixed point, so that a
        trajectory is the same bits on every run (default: the model's
        default, on for FP32).  rebuild_every: steps between Verlet-list
        rebuilds for a batch with a skin (ignored without one)."""
        dev = model.device
        dt_t = model.dtype
        self.model, self.batch, self.dt = model, batch, dt
        self.det = deterministic
        self.every = max(1, int(rebuild_every)) if batch.skin > 0 else 1
        self.nstep = 0
        self.x = torch.tensor(coord, dtype=dt_t, device=dev)
        self.v = torch.tensor(vel, dtype=dt_t, device=dev)
        m = np.array([MASS[int(t)] for t in atype])
        self.minv = torch.tensor(ACC_UNIT / m, dtype=dt_t, device=dev)[:, None]
        self.mass = torch.tensor(m, dtype=torch.float64, device=dev)
        E, F, V = model.step_fused(batch, self.x, self.det)
        self.E, self.F, self.V = E, F, V
        self.graph = None

    def _step(self, rebuild: bool = True):
        h = 0.5 * self.dt
        self.v.add_(self.F * self.minv, alpha=h)
        self.x.add_(self.v, alpha=self.dt)
        E, F, V = self.model.step_fused(self.batch, self.x, self.det, rebuild=rebuild)
        self.v.add_(F * self.minv, alpha=h)
        return E, F, V

    def capture(self):
        # snapshot first: the side stream only waits for work enqueued
        # before wait_stream, so a clone issued after it could read x / v
        # after the warm-up steps on s have already moved them
        x0, v0 = self.x.clone(), self.v.clone()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for k in range(2):
                self._step(rebuild=True)
                if self.every > 1:
                    self._step(rebuild=False)
        torch.cuda.current_stream().wait_stream(s)
        self.x.copy_(x0)
        self.v.copy_(v0)
        self.model.step_fused(self.batch, self.x, self.det)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.E, self.F, self.V = self._step(rebuild=True)
        self.graph_reuse = None
        if self.every > 1:
            self.graph_reuse = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph_reuse):
                self._step(rebuild=False)
        # capture ran nothing: restore the state before the first real step
        # (which rebuilds: the list is made from these coordinates)
        self.x.copy_(x0)
        self.v.copy_(v0)
        self.model.step_fused(self.batch, self.x, self.det)
        self.nstep = 0

    def run(self, nsteps: int):
        """Replay nsteps MD steps: the first of every rebuild_every steps
        rebuilds the list (counting from the state the integrator started
        from, whose forces came from a rebuild)."""
        for _ in range(nsteps):
            self.nstep += 1
            if self.graph_reuse is None or self.nstep % self.every == 0:
                self.graph.replay()
            else:
                self.graph_reuse.replay()

    def total_energy(self) -> float:
        ke = 0.5 * float((self.mass[:, None] * self.v.double() ** 2).sum()) * KE_UNIT
        return float(self.E.sum()) + ke

    def temperature(self) -> float:
        ke = 0.5 * float((self.mass[:, None] * self.v.double() ** 2).sum()) * KE_UNIT
        return 2.0 * ke / (3 * len(self.mass) * KB_EV)
