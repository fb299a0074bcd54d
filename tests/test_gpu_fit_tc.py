"""Tensor-core fitting (tcgen05 kind::f16, scaled FP16 hi/lo split) against the
cuBLAS FP32 path on the same descriptor rows, and the fused step with it
against the FP64 composite.

Stated tolerances: per-atom energy and dE/dD within 1e-5 relative to the
largest magnitude (split products with short tensor-core accumulation
chains; measured 3.0e-6 and 1.2e-6 on this net); forces <= 1e-5 eV/A vs
FP64."""

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
    stat = [water.water_frame(4, 12.42, 4000 + s) for s in range(4)]
    m64 = se_a.build_model(cfg, 29, stat, DEV, torch.float64)
    mk = lambda mode: se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(),
                                    m64.dstd.cpu().numpy(), DEV, torch.float32, m64.tables_np,
                                    m64.infos_np, fit_mode=mode)
    return se_a, cfg, m64, mk, water


def test_tc_fitting_matches_fp32_gemm(setup):
    se_a, cfg, m64, mk, water = setup
    ref, tc = mk("native-fp32"), mk("tc-f16x3")
    frame = water.water_frame(5, 15.525, 8)  # 375 atoms: 125 O, 250 H (ragged 128-blocks)
    bt = tc.batch([frame[1]], frame[2][None])
    br = ref.batch([frame[1]], frame[2][None])
    coord = torch.tensor(frame[0], dtype=torch.float32, device=DEV)
    tc.step_fused(bt, coord)
    ref.step_fused(br, coord)
    torch.cuda.synchronize()
    assert tc._lib.gbdp_fitting_tc_status(
        bt.tc_ws.data_ptr(), bt.nrows_total, torch.cuda.current_stream().cuda_stream) == 0
    for t, ((s_t, n_t), (s_r, n_r)) in enumerate(zip(bt.type_rows, br.type_rows)):
        assert n_t == n_r
        e_tc, e_ref = bt.ae[s_t:s_t + n_t], br.ae[s_r:s_r + n_r]
        g_tc, g_ref = bt.dD[s_t:s_t + n_t], br.dD[s_r:s_r + n_r]
        err_e = float((e_tc - e_ref).abs().max()) / float(e_ref.abs().max())
        err_g = float((g_tc - g_ref).abs().max()) / float(g_ref.abs().max())
        print(f"type {t}: relative max error e {err_e:.3e}, dE/dD {err_g:.3e}")
        assert err_e <= 1e-5 and err_g <= 1e-5, (t, err_e, err_g)
        if t == 0:  # padding rows of the first block carry no energy
            assert float(bt.ae[s_t + n_t:bt.type_rows[1][0]].abs().max()) == 0.0


def test_tc_fused_step_vs_fp64(setup):
    import composite

    se_a, cfg, m64, mk, water = setup
    tc = mk("tc-f16x3")
    frame = water.water_frame(4, 12.42, 5)
    b = tc.batch([frame[1]], frame[2][None])
    E, F, V = tc.step_fused(b, torch.tensor(frame[0], dtype=torch.float32, device=DEV))
    Er, Fr, Vr, _ = composite.energy_force_virial(cfg, m64.params_np, m64.davg.cpu().numpy(),
                                                  m64.dstd.cpu().numpy(), *frame, m64.tables_np,
                                                  m64.infos_np)
    assert np.abs(F.cpu().numpy().astype(np.float64) - Fr).max() <= 1e-5
    assert abs(float(E[0]) - Er) / len(frame[1]) <= 1e-6
    assert np.abs(V[0].cpu().numpy() - Vr).max() <= 1e-3


def test_persistent_short_k_layers_equal_per_tile(setup):
    """The K-240 layers on the persistent kernel (forced with a threshold of
    one tile per SM, 128-wide tiles) give the same bits as one CTA per tile
    (80-wide tiles): the same MMAs into the same accumulators and the same
    epilogue per column, on a ragged batch of two type blocks.  The atom
    energies sum F3's per-tile partials, two of them against three, so they
    agree to rounding only."""
    se_a, cfg, m64, mk, water = setup
    tc = mk("tc-f16x3")
    frames = water.ragged_frames(12, seed=31, lo=40, hi=300)
    b = tc.batch([f[1] for f in frames], np.stack([f[2] for f in frames]))
    coord = torch.tensor(np.concatenate([f[0] for f in frames]), dtype=torch.float32, device=DEV)
    lib = tc._lib
    out = []
    try:
        for thr in (1 << 20, 1):
            lib.gbdp_fitting_tc_set_persistent_min_tiles(thr)
            E, F, V = tc.step_fused(b, coord)
            torch.cuda.synchronize()
            assert lib.gbdp_fitting_tc_status(b.tc_ws.data_ptr(), b.nrows_total,
                                              torch.cuda.current_stream().cuda_stream) == 0
            out.append((b.ae.clone(), b.dD.clone(), F.clone(), V.clone()))
    finally:
        lib.gbdp_fitting_tc_set_persistent_min_tiles(32)
    torch.testing.assert_close(out[0][0], out[1][0], rtol=1e-6, atol=1e-6)
    for x, y in zip(out[0][1:], out[1][1:]):
        assert torch.equal(x, y)
