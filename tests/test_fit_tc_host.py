"""Host side of the tensor-core fitting: the power-of-two scales and FP16
hi / lo weight images (dpmd_public_gb300.se_a), and the activation bounds
the scales come from, checked against the fitting net's own forward and
backward in FP64 on random and saturating inputs."""

import importlib
import math

import numpy as np
import pytest
import torch


def _se_a(gb):
    return importlib.import_module("dpmd_public_gb300.se_a")


def test_f16_scale_brackets_the_bound(gb):
    se_a = _se_a(gb)
    for b in [1e-30, 3.3e-9, 2.0 ** -14, 0.37, 1.0, 1.01, 2.0, 255.9, 65504.0, 1e12, 3e37]:
        sc = se_a._f16_scale(b)
        assert math.frexp(sc)[0] == 0.5  # a power of two
        assert 2.0 ** 14 <= b * sc < 2.0 ** 15
    for b in [0.0, -1.0, float("inf"), float("nan")]:
        assert se_a._f16_scale(b) == 1.0


def test_split_rows_reconstruct_to_fp32_level(gb):
    se_a = _se_a(gb)
    g = torch.Generator().manual_seed(3)
    mags = torch.logspace(-6, 3, 40)
    m = (torch.randn(40, 1600, generator=g) * mags[:, None]).float()
    m[5, :] = 0.0
    m[7, 100:] = 0.0
    hi, lo, inv = se_a._split_f16_rows(m)
    assert hi.dtype == torch.float16 and lo.dtype == torch.float16
    assert torch.isfinite(hi).all() and torch.isfinite(lo).all()
    assert float(hi.float().abs().max()) < 2.0 ** 15
    # inverse scales are powers of two; the reconstruction holds each row to
    # 2^-21 of its largest magnitude
    assert np.all(np.frexp(inv.numpy())[0] == 0.5)
    rec = (hi.double() + lo.double()) * inv.double()[:, None]
    err = (rec - m.double()).abs().amax(dim=1)
    rowmax = m.double().abs().amax(dim=1)
    assert torch.all(err <= 2.0 ** -21 * rowmax)
    assert float(err[5]) == 0.0


def _net(gb, seed):
    mdl = importlib.import_module("dpmd_public_gb300.model")
    cfg = mdl.SeAConfig()
    p = mdl.init_params(cfg, seed)
    out = []
    for f in p["fit"]:
        hid = [(torch.tensor(L["w"], dtype=torch.float32), torch.tensor(L["b"], dtype=torch.float32),
                None if L["idt"] is None else torch.tensor(L["idt"], dtype=torch.float32), L["skip"])
               for L in f["hidden"]]
        out.append((hid, torch.tensor(f["final"]["w"][:, 0], dtype=torch.float32)))
    return out


def _activations(hidden, wo, D):
    """H1, H2, GZ3, GZ2, GZ1 of the fitting net on rows D (FP64)."""
    (w1, b1, _, _), (w2, b2, i2, _), (w3, b3, i3, _) = [
        tuple(x.double() if isinstance(x, torch.Tensor) else x for x in L) for L in hidden]
    wo = wo.double()
    t1 = torch.tanh(D @ w1 + b1)
    t2 = torch.tanh(t1 @ w2 + b2)
    h2 = t2 * i2 + t1
    t3 = torch.tanh(h2 @ w3 + b3)
    gz3 = wo * i3 * (1 - t3 * t3)
    g2 = gz3 @ w3.T + wo
    gz2 = g2 * i2 * (1 - t2 * t2)
    g1 = gz2 @ w2.T + g2
    gz1 = g1 * (1 - t1 * t1)
    return [t1, h2, gz3, gz2, gz1]


@pytest.mark.parametrize("seed", [1, 2])
def test_activation_scales_bound_the_activations(gb, seed):
    se_a = _se_a(gb)
    g = torch.Generator().manual_seed(seed)
    for hidden, wo in _net(gb, seed):
        sc = se_a._fit_tc_act_scales(hidden, wo)
        assert all(math.frexp(s)[0] == 0.5 for s in sc)
        # typical rows, rows that saturate every tanh, and rows near zero
        D = torch.cat([torch.randn(512, 1600, generator=g, dtype=torch.float64),
                       1e3 * torch.randn(64, 1600, generator=g, dtype=torch.float64),
                       1e-4 * torch.randn(64, 1600, generator=g, dtype=torch.float64)])
        for a, s in zip(_activations(hidden, wo, D), sc):
            peak = float(a.abs().max()) * s
            assert peak < 2.0 ** 15  # no FP16 part can overflow
            assert peak >= 2.0 ** 3  # and the bound is not loose enough to cost precision
