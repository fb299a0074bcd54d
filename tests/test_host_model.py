"""Host-side logic on CPU: the synthetic water generator, model parameters,
descriptor statistics, compression tables, and the FP64 CPU composite the
GPU forms are checked against (validated here by finite differences)."""

import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def m(gb):
    return (importlib.import_module("dpmd_public_gb300.model"),
            importlib.import_module("dpmd_public_gb300.water"))


def test_water_geometry(m):
    mdl, water = m
    c, t, b = water.water_frame(4, 12.42, 3, jitter=0.0)
    assert c.shape == (192, 3) and list(t[:3]) == [0, 1, 1]
    L = b[0]
    mol = c.reshape(-1, 3, 3)
    d = mol[:, 1:] - mol[:, :1]
    d -= L * np.round(d / L)
    r = np.linalg.norm(d, axis=-1)
    np.testing.assert_allclose(r, 0.9572, atol=1e-9)
    cosang = (d[:, 0] * d[:, 1]).sum(-1) / (r[:, 0] * r[:, 1])
    np.testing.assert_allclose(np.degrees(np.arccos(cosang)), 104.52, atol=1e-7)
    assert (c >= 0).all() and (c < L).all()
    # same seed, same frame
    np.testing.assert_array_equal(water.water_frame(4, 12.42, 3)[0], water.water_frame(4, 12.42, 3)[0])


def test_ragged_frames_density(m):
    mdl, water = m
    fr = water.ragged_frames(6, seed=1, lo=8, hi=512)
    for c, t, b in fr:
        n = len(t) // 3
        assert 8 <= n <= 512
        assert abs(b[0] ** 3 / n - water.VOL_PER_MOLECULE) < 1e-9


def test_table_reproduces_embedding(m):
    """At every grid node the row polynomial equals the net's value; between
    nodes the quintic Hermite error is tiny."""
    mdl, water = m
    cfg = mdl.SeAConfig()
    p = mdl.init_params(cfg, 3)
    davg = np.zeros((2, cfg.nnei * 4))
    dstd = np.ones((2, cfg.nnei * 4))
    davg[:, 0::4] = 0.05
    dstd[:, 0::4] = 0.13
    tabs, infos = mdl.build_tables(p, davg, dstd, 0.8, cfg)
    lo, up, mx, s0, s1 = infos[0][:5]
    M = cfg.neuron[-1]
    for x in (-0.37, 0.123, 2.71, float(up) + 0.33):
        if x < up:
            idx = int((x - lo) / s0)
            dx = x - (idx * s0 + lo)
        else:
            first = int((up - lo) / s0)
            idx = first + int((x - up) / s1)
            dx = x - ((idx - first) * s1 + up)
        a = tabs[0][idx].reshape(M, 6)
        val = a[:, 0] + (a[:, 1] + (a[:, 2] + (a[:, 3] + (a[:, 4] + a[:, 5] * dx) * dx) * dx) * dx) * dx
        exact = mdl.embedding_value_and_derivs(p["emb"][0], np.array([x]))[0][0]
        np.testing.assert_allclose(val, exact, atol=1e-9)


def test_stats_protection_and_layout(m):
    mdl, water = m
    cfg = mdl.SeAConfig()
    em = np.zeros((4, cfg.nnei, 4))
    em[:, :10, 0] = 0.5
    davg, dstd = mdl.stats_from_env([em], [np.array([0, 0, 1, 1])], cfg)
    assert davg.shape == (2, cfg.nnei * 4)
    np.testing.assert_allclose(davg[:, 0::4], 0.5 * 10 / cfg.nnei)
    assert (davg[:, 1::4] == 0).all()
    assert (dstd[:, 1::4] == 1e-2).all()  # zero spread -> protection


def test_composite_force_is_minus_energy_gradient(m):
    """FD check of the CPU composite (compressed and plain), the reference
    used by every end-to-end GPU test: h = 1e-5 A central differences."""
    import composite

    mdl, water = m
    cfg = mdl.SeAConfig()
    p = mdl.init_params(cfg, 1)
    davg = np.zeros((2, cfg.nnei * 4))
    dstd = np.ones((2, cfg.nnei * 4))
    davg[:, 0::4] = 0.049
    dstd[:, 0::4] = 0.13
    dstd[:, 1::4] = dstd[:, 2::4] = dstd[:, 3::4] = 0.08
    tabs, infos = mdl.build_tables(p, davg, dstd, 0.77, cfg)
    c, t, b = water.water_frame(2, 6.2, 7)
    for tb, inf in ((None, None), (tabs, infos)):
        E, F, V, _ = composite.energy_force_virial(cfg, p, davg, dstd, c, t, b, tb, inf)
        h = 1e-5
        for a, d in ((0, 0), (5, 1), (13, 2)):
            cp, cm = c.copy(), c.copy()
            cp[a, d] += h
            cm[a, d] -= h
            Ep = composite.energy_force_virial(cfg, p, davg, dstd, cp, t, b, tb, inf)[0]
            Em = composite.energy_force_virial(cfg, p, davg, dstd, cm, t, b, tb, inf)[0]
            assert abs(-(Ep - Em) / (2 * h) - F[a, d]) < 1e-8


@pytest.mark.parametrize("tag", ["small", "bench_one_side", "bench_pair"])
def test_tables_match_reference_dptabulate(m, tag):
    """build_tables against tables the reference's own DPTabulate built
    (tests/golden/ref_tabulate.npz, made by make_golden.py from the
    reference sources) for the same seeded nets and statistics: the range
    (lower, upper, row count) exactly; each row's value, slope and curvature
    coefficients to 1e-13 of their column's scale, and the row polynomial
    and its slope inside the interval to 1e-13 / 1e-11 (the whole table for
    the small net, sampled rows and per-column sums for the 25-50-100
    nets)."""
    import dataclasses
    import os

    mdl, water = m
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_tabulate.npz"))
    base = mdl.SeAConfig()
    cfg = {"small": dataclasses.replace(base, neuron=(2, 4, 8), stride0=0.1, stride1=1.0),
           "bench_one_side": base,
           "bench_pair": dataclasses.replace(base, type_one_side=False)}[tag]
    params = mdl.init_params(cfg, int(g[f"{tag}_seed"]))
    tabs, infos = mdl.build_tables(params, g[f"{tag}_davg"], g[f"{tag}_dstd"],
                                   float(g[f"{tag}_rmin"]), cfg)
    names = [str(x) for x in g[f"{tag}_nets"]]
    nt = cfg.ntypes
    for k, name in enumerate(names):
        # the reference's table k: filter_-1_net_{tj} (one side) or
        # filter_{ti}_net_{tj}; ours are indexed tj (one side) or tj * nt + ti
        if cfg.type_one_side:
            ours = int(name.split("_")[-1])
        else:
            ti, tj = int(name.split("_")[1]), int(name.split("_")[3])
            ours = tj * nt + ti
        t, info = tabs[ours], infos[ours]
        assert info[0] == g[f"{tag}_{k}_lower"] and info[1] == g[f"{tag}_{k}_upper"]
        assert t.shape[0] == int(g[f"{tag}_{k}_nspline"])
        if f"{tag}_{k}_table" in g:
            ref = g[f"{tag}_{k}_table"]
            rows = np.arange(t.shape[0])
        else:
            rows = g[f"{tag}_{k}_rows"]
            ref = g[f"{tag}_{k}_sample"]
            t = t[rows]
        a, b = t.reshape(len(rows), -1, 6), ref.reshape(len(rows), -1, 6)
        # value, slope and curvature at the row's first node
        scale = np.abs(b).max(axis=(0, 1))
        for c in range(3):
            assert np.abs(a[..., c] - b[..., c]).max() <= 1e-13 * scale[c], (name, c)
        # the interpolant and its slope inside each interval (the higher
        # coefficients carry the nodes' rounding amplified by 1 / stride^n in
        # any evaluation order; their effect on the polynomial is what counts)
        n0 = int((info[1] - info[0]) / cfg.stride0)
        tt = np.where(rows < n0, cfg.stride0, cfg.stride1)[:, None]
        vmax, dmax = np.abs(b[..., 0]).max(), np.abs(b[..., 1]).max()
        for f in (0.25, 0.5, 0.75, 1.0):
            u = f * tt
            pa = sum(a[..., c] * u ** c for c in range(6))
            pb = sum(b[..., c] * u ** c for c in range(6))
            da = sum(c * a[..., c] * u ** (c - 1) for c in range(1, 6))
            db = sum(c * b[..., c] * u ** (c - 1) for c in range(1, 6))
            assert np.abs(pa - pb).max() <= 1e-13 * vmax, (name, f)
            assert np.abs(da - db).max() <= 1e-11 * dmax, (name, f)
        colsum = np.abs(tabs[ours]).reshape(tabs[ours].shape[0], -1, 6).sum(axis=(0, 1))
        np.testing.assert_allclose(colsum[:3], g[f"{tag}_{k}_colsum"][:3], rtol=1e-13)


def test_batch_rejects_atom_types_outside_the_model(gb):
    """A fused-step batch gives every atom a row of D by its type; a type
    outside [0, ntypes) is rejected before any device work."""
    import importlib

    import pytest

    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")

    class _Model:  # only what Batch reads before the check
        cfg = mdl.SeAConfig()
        device = "cpu"
        dtype = None

    box = np.diag([12.0] * 3).reshape(1, 9)
    for bad in ([0, 1, -1], [0, 2, 1]):
        with pytest.raises(ValueError, match="atom types"):
            se_a.Batch(_Model(), [np.array(bad, np.int32)], box)
