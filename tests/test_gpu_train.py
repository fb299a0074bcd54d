"""Training step (force-loss double backward) and finite-difference checks,
FP64 on the 24-atom (8 H2O) frame in a 6.2 A box:
  * forces of the fused and operator forms = -dE/dx by central differences
    with h = 1e-5 A (|diff| <= 1e-7 eV/A);
  * gradients of the EnergyStdLoss (pref_e 0.02, pref_f 1000, pref_v 0.02)
    wrt fitting parameters, through tabulate grad-grad and prod_force_grad,
    = central differences of the loss (relative 1e-5)."""

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
    stat = [water.water_frame(4, 12.42, 2000 + s) for s in range(4)]
    m = se_a.build_model(cfg, 17, stat, DEV, torch.float64)
    frame = water.water_frame(2, 6.2, 31)
    return se_a, m, frame


def test_forces_are_minus_energy_gradient(setup):
    se_a, m, (c, t, b) = setup
    batch = m.batch([t], b[None])
    base = torch.tensor(c, dtype=torch.float64, device=DEV)
    for form in ("fused", "ops"):
        def energy(x):
            if form == "fused":
                return float(m.step_fused(batch, x)[0][0])
            return float(m.step_ops(batch, x)[0][0])
        if form == "fused":
            F = m.step_fused(batch, base)[1].clone().cpu().numpy()
        else:
            F = m.step_ops(batch, base)[1].detach().cpu().numpy()
        h = 1e-5
        for a, d in ((0, 0), (4, 1), (11, 2), (23, 0)):
            xp, xm = base.clone(), base.clone()
            xp[a, d] += h
            xm[a, d] -= h
            fd = -(energy(xp) - energy(xm)) / (2 * h)
            assert abs(fd - F[a, d]) < 1e-7, (form, a, d, fd, F[a, d])


def test_force_loss_gradient_double_backward(setup):
    se_a, m, (c, t, b) = setup
    batch = m.batch([t], b[None])
    x = torch.tensor(c, dtype=torch.float64, device=DEV)
    tr = se_a.Trainable(m)
    E0, F0, V0 = tr.energy_force_virial(batch, x)
    rng = np.random.default_rng(0)
    E_ref = (E0.detach() + 0.3).detach()
    F_ref = (F0.detach() + torch.tensor(rng.normal(0, 0.05, F0.shape), device=DEV)).detach()
    V_ref = (V0.detach() - 0.2).detach()

    def loss():
        E, F, V = tr.energy_force_virial(batch, x)
        return se_a.energy_std_loss(E, F, V, E_ref, F_ref, V_ref, len(t))

    L = loss()
    grads = torch.autograd.grad(L, tr.params)
    checks = [(0, (3, 5)), (1, (7,)), (len(tr.params) - 2, (11, 0)), (2, (13, 7))]
    for pi, idx in checks:
        p = tr.params[pi]
        g = grads[pi][idx].item()
        h = 1e-6
        with torch.no_grad():
            p[idx] += h
        lp = loss().item()
        with torch.no_grad():
            p[idx] -= 2 * h
        lm = loss().item()
        with torch.no_grad():
            p[idx] += h
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g) <= 1e-5 * max(1.0, abs(fd)), (pi, idx, fd, g)


def test_bf16_fitting_gemms_training_step(gb):
    """The training step on a batch of 8 seeded 192-atom frames (FP32 model)
    with the fitting GEMMs in BF16 (FP32 accumulation, products rounded to
    BF16) against FP32.  Stated BF16 tolerances: loss within 1e-3 relative;
    the fitting-parameter gradient within 0.2 relative L2 and at cosine
    similarity >= 0.99 (a force-loss gradient of perturbed labels is a small
    residual, and every double-backward product is BF16-rounded; measured
    values printed)."""
    gb.load_library()
    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")
    water = importlib.import_module("dpmd_public_gb300.water")
    cfg = mdl.SeAConfig()
    stat = [water.water_frame(4, 12.42, 2000 + s) for s in range(4)]
    m64 = se_a.build_model(cfg, 17, stat, DEV, torch.float64)
    m = se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), DEV,
                      torch.float32, m64.tables_np, m64.infos_np)
    frames = [water.water_frame(4, 12.42, 40 + k) for k in range(8)]
    batch = m.batch([f[1] for f in frames], np.stack([f[2] for f in frames]))
    x = torch.tensor(np.concatenate([f[0] for f in frames]), dtype=torch.float32, device=DEV)
    E0, F0, V0 = se_a.Trainable(m).energy_force_virial(batch, x)
    gen = torch.Generator(device=DEV).manual_seed(3)
    E_ref = (E0 + 0.1 * torch.randn(E0.shape, generator=gen, device=DEV)).detach()
    F_ref = (F0 + 0.05 * torch.randn(F0.shape, generator=gen, device=DEV)).detach()
    V_ref = (V0 + 0.1 * torch.randn(V0.shape, generator=gen, device=DEV)).detach()
    out = {}
    for gemm in ("fp32", "bf16"):
        tr = se_a.Trainable(m, gemm)
        E, F, V = tr.energy_force_virial(batch, x)
        L = se_a.energy_std_loss(E, F, V, E_ref, F_ref, V_ref, 192)
        g = torch.autograd.grad(L, tr.params)
        out[gemm] = (float(L), torch.cat([t.reshape(-1) for t in g]))
    dl = abs(out["bf16"][0] - out["fp32"][0]) / abs(out["fp32"][0])
    g16, g32 = out["bf16"][1].double(), out["fp32"][1].double()
    dg = float((g16 - g32).norm() / g32.norm())
    cos = float(g16 @ g32 / (g16.norm() * g32.norm()))
    print(f"BF16 fitting GEMMs: loss rel diff {dl:.3e}, gradient rel L2 diff {dg:.3e}, "
          f"cosine {cos:.6f}")
    assert dl <= 1e-3 and dg <= 0.2 and cos >= 0.99
