"""The fused, operator and plain forms on se_e2_a configurations other than
the 25-50-100 / sel [46, 92] water model: other embedding widths (M = 16,
32, 48, 64, 128 select the other chunk / tail instantiations of the fused
kernels), one net per (neighbour, centre) type pair, three atom types, a
shorter cutoff, other fitting widths, and neighbour lists truncated at sel
(water has about 30 O and 60 H neighbours within 6 A).

Stated tolerances against the FP64 CPU composite (oracle/composite.py):
  fp64 GPU: |dF| <= 1e-9 eV/A, |dE| / natoms <= 1e-10 eV, |dV| <= 1e-8 eV
  fp32 GPU: |dF| <= 1e-5 eV/A, |dE| / natoms <= 1e-6 eV, |dV| <= 1e-3 eV
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"

CONFIGS = {
    # pair nets (4 tables), M = 64: two full 32-wide output chunks; lists truncated
    "pair_m64": dict(neuron=(16, 32, 64), sel=(20, 40), type_one_side=False, fitting=(120, 120, 120)),
    # M = 48: one chunk and a 16-wide tail; rcut 5 with a 1 A smoothing band
    "tail_m48": dict(neuron=(12, 24, 48), sel=(30, 60), rcut=5.0, rcut_smth=1.0, fitting=(64, 64)),
    # M = 128, the widest the fused kernels take; short lists
    "wide_m128": dict(neuron=(32, 64, 128), sel=(12, 24), fitting=(240, 240, 240)),
    # M = 16 = axis_neuron, the narrowest; pair nets; a single fitting layer
    "narrow_m16": dict(neuron=(4, 8, 16), sel=(46, 92), type_one_side=False, fitting=(32,)),
    # three atom types (every third H relabelled), nine pair nets, M = 32
    "three_types": dict(ntypes=3, neuron=(8, 16, 32), sel=(30, 40, 30), type_one_side=False,
                        fitting=(50, 50)),
}

TOL = {torch.float64: (1e-9, 1e-10, 1e-8), torch.float32: (1e-5, 1e-6, 1e-3)}


@pytest.fixture(scope="module")
def mods(gb):
    gb.load_library()
    import importlib

    return (importlib.import_module("dpmd_public_gb300.se_a"),
            importlib.import_module("dpmd_public_gb300.model"),
            importlib.import_module("dpmd_public_gb300.water"))


def _frame(water, ntypes, seed):
    c, t, b = water.water_frame(4, 12.42, seed)
    t = np.asarray(t, dtype=np.int32).copy()
    if ntypes == 3:
        h = np.flatnonzero(t == 1)
        t[h[::3]] = 2
    return c, t, b


_BUILT = {}


def _models(mods, name):
    if name not in _BUILT:
        se_a, mdl, water = mods
        cfg = mdl.SeAConfig(**CONFIGS[name])
        stat = [_frame(water, cfg.ntypes, 2000 + s) for s in range(3)]
        m64 = se_a.build_model(cfg, 11, stat, DEV, torch.float64)
        m32 = se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), DEV,
                            torch.float32, m64.tables_np, m64.infos_np)
        _BUILT[name] = (cfg, m64, m32)
    return _BUILT[name]


_REF = {}


def _ref(cfg, m64, frame, name, compressed):
    import composite

    key = (name, compressed)
    if key not in _REF:
        c, t, b = frame
        _REF[key] = composite.energy_force_virial(
            cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), c, t, b,
            m64.tables_np if compressed else None, m64.infos_np if compressed else None)
    return _REF[key]


def _check(E, F, V, ref, natoms, dtype):
    ft, et, vt = TOL[dtype]
    Er, Fr, Vr, _ = ref
    F = F.detach().cpu().numpy().astype(np.float64)
    assert abs(float(E) - Er) / natoms <= et, (float(E), Er)
    assert np.abs(F - Fr).max() <= ft, np.abs(F - Fr).max()
    assert np.abs(V.cpu().numpy() - Vr).max() <= vt, np.abs(V.cpu().numpy() - Vr).max()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("form", ["fused", "fused-atomic", "ops", "plain"])
@pytest.mark.parametrize("name", list(CONFIGS))
def test_config_forms_vs_fp64_composite(mods, name, form, dtype):
    se_a, mdl, water = mods
    cfg, m64, m32 = _models(mods, name)
    m = m64 if dtype == torch.float64 else m32
    frame = _frame(water, cfg.ntypes, 21)
    b = m.batch([frame[1]], frame[2][None])
    coord = torch.tensor(frame[0], dtype=dtype, device=DEV)
    if form.startswith("fused"):
        E, F, V = m.step_fused(b, coord, deterministic=(form == "fused"))
        assert b.status() == 0
    else:
        E, F, V = m.step_ops(b, coord, compressed=(form == "ops"))
    ref = _ref(cfg, m64, frame, name, compressed=(form != "plain"))
    _check(E[0].item(), F, V[0], ref, len(frame[1]), dtype)


@pytest.mark.parametrize("name", ["pair_m64", "three_types"])
def test_config_ragged_batch(mods, name):
    """Frames of different sizes (and one with no atoms of the last type)
    packed into one batch give each frame's own single-frame result."""
    se_a, mdl, water = mods
    cfg, m64, m32 = _models(mods, name)
    frames = [water.water_frame(3, 9.3, 31), _frame(water, cfg.ntypes, 32),
              water.water_frame(2, 6.3, 33, n_mol=5)]
    b = m32.batch([f[1] for f in frames], np.stack([f[2] for f in frames]))
    coord = torch.tensor(np.concatenate([f[0] for f in frames]), dtype=torch.float32, device=DEV)
    E, F, V = (x.clone() for x in m32.step_fused(b, coord))
    assert b.status() == 0
    off = 0
    for i, f in enumerate(frames):
        n = len(f[1])
        b1 = m32.batch([f[1]], f[2][None])
        E1, F1, V1 = m32.step_fused(b1, torch.tensor(f[0], dtype=torch.float32, device=DEV))
        assert abs(float(E[i]) - float(E1[0])) <= 1e-6 * n
        assert float((F[off:off + n] - F1).abs().max()) <= 1e-6
        assert float((V[i] - V1[0]).abs().max()) <= 1e-4
        off += n
