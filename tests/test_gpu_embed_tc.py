"""BF16 tensor-core embedding of the uncompressed se_e2_a descriptor
(csrc/embed_tc.cu) against the FP32 torch embedding of the same model, and
the whole tensor-core plain step against the FP64 CPU composite.

Stated tolerances (BF16 MMA operands with FP32 accumulation, tanh.approx;
relative to the largest magnitude of the reference):
  X and D:            max |diff| <= 1e-2 max |ref|
  dE/d(env matrix):   max |diff| <= 2e-2 max |ref|
  plain-tc step vs FP64: |dF| <= 2e-2 eV/A, |dE| / natoms <= 1e-3 eV
The measured errors are printed."""

import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def setup(gb):
    gb.load_library()
    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")
    water = importlib.import_module("dpmd_public_gb300.water")
    cfg = mdl.SeAConfig()
    stat = [water.water_frame(4, 12.42, 1000 + s) for s in range(4)]
    m64 = se_a.build_model(cfg, 7, stat, DEV, torch.float64)
    args = (cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), DEV, torch.float32)
    return se_a, water, cfg, m64, se_a.SeAModel(*args), se_a.SeAModel(*args, fit_mode="tc-f16x3")


def _ref_x(model, em, atype):
    """X [n, 4, M] of the FP32 torch embedding (the plain form's nets)."""
    cfg = model.cfg
    n, sec, M = em.shape[0], cfg.sec, cfg.neuron[-1]
    X = torch.zeros((n, 4, M), dtype=em.dtype, device=em.device)
    for tj in range(cfg.ntypes):
        for ti in ([None] if cfg.type_one_side else range(cfg.ntypes)):
            k = tj if cfg.type_one_side else tj * cfg.ntypes + ti
            rows = torch.arange(n, device=em.device) if ti is None else torch.nonzero(atype == ti)[:, 0]
            rr = em[rows, sec[tj]:sec[tj + 1], :]
            g = rr[:, :, :1]
            for w, b, skip in model.emb[k]:
                y = torch.tanh(g @ w + b)
                if skip == "same":
                    y = y + g
                elif skip == "double":
                    y = y + torch.cat([g, g], -1)
                g = y
            X = X.index_add(0, rows, rr.transpose(1, 2) @ g)
    return X / cfg.nnei


def _case(setup, mdl_idx, seed=5, n=4, L=12.42):
    se_a, water, cfg, m64, m32, m32tc = setup
    m = (m32, m32tc)[mdl_idx]
    c, t, b = water.water_frame(n, L, seed)
    batch = m.batch([t], b[None])
    coord = torch.tensor(c, dtype=torch.float32, device=DEV)
    batch.ensure_plain_tc(m)
    env = se_a.env_mat_packed(batch.plan, coord, batch.atype, m.davg, m.dstd, cfg.rcut_smth,
                              list(cfg.sel), out=batch.env_full)
    return m, batch, env, (c, t, b)


@pytest.mark.parametrize("mdl_idx", [0, 1])
def test_forward_x_and_d(setup, mdl_idx):
    m, batch, env, _ = _case(setup, mdl_idx)
    cfg = m.cfg
    m.embed_tc_forward(batch, env.em)
    torch.cuda.synchronize()
    assert int(batch.emb_status.item()) == 0
    Xr = _ref_x(m, env.em, batch.atype)
    ex = float((batch.X - Xr).abs().max() / Xr.abs().max())
    A = cfg.axis_neuron
    Dr = torch.einsum("ncm,nca->nma", Xr, Xr[:, :, :A]).reshape(batch.nloc, -1)
    D = batch.descriptor_rows()[batch.drow.long()]
    ed = float((D - Dr).abs().max() / Dr.abs().max())
    print(f"X rel err {ex:.3e}, D rel err {ed:.3e}")
    assert ex <= 1e-2 and ed <= 1e-2


def test_backward_env_gradient(setup):
    m, batch, env, _ = _case(setup, 0, seed=8)
    cfg = m.cfg
    m.embed_tc_forward(batch, env.em)
    gen = torch.Generator(device=DEV).manual_seed(2)
    batch.dD.copy_(torch.randn(batch.dD.shape, generator=gen, device=DEV))
    net = m.embed_tc_backward(batch, env.em)
    torch.cuda.synchronize()
    assert int(batch.emb_status.item()) == 0
    em = env.em.clone().requires_grad_(True)
    Xr = _ref_x(m, em, batch.atype)
    A = cfg.axis_neuron
    Dr = torch.einsum("ncm,nca->nma", Xr, Xr[:, :, :A]).reshape(batch.nloc, -1)
    g = torch.autograd.grad(Dr, em, grad_outputs=batch.dD[batch.drow.long()])[0]
    e = float((net - g).abs().max() / g.abs().max())
    print(f"dE/d(env) rel err {e:.3e}")
    assert e <= 2e-2


@pytest.mark.parametrize("mdl_idx", [0, 1])
def test_plain_tc_step_vs_fp64(setup, mdl_idx):
    import composite

    se_a, water, cfg, m64, m32, m32tc = setup
    m, batch, env, (c, t, b) = _case(setup, mdl_idx, seed=11)
    E, F, V = m.step_plain_tc(batch, torch.tensor(c, dtype=torch.float32, device=DEV))
    torch.cuda.synchronize()
    assert int(batch.emb_status.item()) == 0
    Er, Fr, Vr, _ = composite.energy_force_virial(cfg, m64.params_np, m64.davg.cpu().numpy(),
                                                  m64.dstd.cpu().numpy(), c, t, b, None, None)
    ef = float(np.abs(F.cpu().numpy().astype(np.float64) - Fr).max())
    ee = abs(float(E[0]) - Er) / len(t)
    ev = float(np.abs(V[0].cpu().numpy() - Vr).max())
    print(f"plain-tc vs FP64: |dF| {ef:.3e} eV/A (max |F| {np.abs(Fr).max():.3f}), "
          f"|dE|/N {ee:.3e} eV, |dV| {ev:.3e} eV")
    assert ef <= 2e-2 and ee <= 1e-3
