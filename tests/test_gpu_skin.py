"""The Verlet-list (skin) form of the env pipeline and of the MD step.

After a rebuild at rcut + skin, the atoms move by up to 0.6 A (less than
half the 2 A skin) and the list is reused: the formatted list equals, bit
for bit, the reference's formatting (oracle format_nlist: build_nlist_cpu +
format_nlist_cpu) of the extended coordinates the step used, the ghosts
refreshed from their atoms.  In fp64 it also equals a fresh build's at the
new coordinates element by element, with the env rows within 1e-12 (values)
and 1e-10 (derivative rows: a refreshed ghost coordinate, coord + shift,
rounds differently from a freshly built one, coord - image vector, and the
derivative rows amplify that).  In fp32 that rounding difference is large
enough to swap neighbours whose float r^2 are within an ulp, so the fp32
check is the oracle's formatting alone.  The fused step on a reused list
gives the energy, forces and virial of a fresh step; NVE with a rebuild
every 10 steps follows the trajectory that rebuilds at every step."""

import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
SEL = [46, 92]
NNEI = sum(SEL)


@pytest.fixture(scope="module")
def mods(gb):
    gb.load_library()
    return (importlib.import_module("dpmd_public_gb300.se_a"),
            importlib.import_module("dpmd_public_gb300.model"),
            importlib.import_module("dpmd_public_gb300.water"),
            importlib.import_module("dpmd_public_gb300.ops"))


def _stats(seed=0):
    rng = np.random.default_rng(seed)
    avg = np.zeros((2, NNEI * 4))
    avg[:, 0::4] = rng.uniform(0.05, 0.15, (2, NNEI))
    std = np.ones((2, NNEI * 4))
    std[:, 0::4] = rng.uniform(0.1, 0.2, (2, NNEI))
    std[:, 1::4] = std[:, 2::4] = std[:, 3::4] = rng.uniform(0.05, 0.1, (2, NNEI))
    return avg, std


def _frames(water):
    fr = [water.water_frame(4, 12.42, 301), water.water_frame(5, 15.525, 302)]
    return fr + water.ragged_frames(2, seed=303, lo=20, hi=80)


def _displace(c, seed, amp=0.6):
    d = np.random.default_rng(seed).normal(0, 0.25, c.shape)
    n = np.linalg.norm(d, axis=1, keepdims=True)
    return c + d * np.minimum(1.0, amp / np.maximum(n, 1e-12))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_reused_list_matches_fresh_build(gb, oracle, mods, dtype):
    se_a, mdl, water, ops = mods
    frames = _frames(water)
    avg_n, std_n = _stats()
    avg = torch.tensor(avg_n, dtype=dtype, device=DEV)
    std = torch.tensor(std_n, dtype=dtype, device=DEV)
    nl = [len(f[1]) for f in frames]
    boxes = np.stack([f[2] for f in frames])
    t = torch.tensor(np.concatenate([f[1] for f in frames]), dtype=torch.int32, device=DEV)
    c0 = np.concatenate([f[0] for f in frames])
    skin_plan = gb.NeighborPlan(nl, boxes, 8.0, DEV, dtype)
    vl = ops.VerletList(skin_plan)
    n = skin_plan.nloc_total
    out = ops.EnvMatResult()
    out.em = torch.empty((n, NNEI, 4), dtype=dtype, device=DEV)
    out.em_deriv = torch.empty((n, NNEI, 4, 3), dtype=dtype, device=DEV)
    out.rij = torch.empty((n, NNEI, 3), dtype=dtype, device=DEV)
    out.nlist = torch.empty((n, NNEI), dtype=torch.int32, device=DEV)
    out.nlist_ext = torch.empty((n, NNEI), dtype=torch.int32, device=DEV)
    out.ext_coord = torch.empty((skin_plan.ext_total, 3), dtype=dtype, device=DEV)
    out.ext_type = torch.empty((skin_plan.ext_total,), dtype=torch.int32, device=DEV)
    out.ext_map = torch.empty((skin_plan.ext_total,), dtype=torch.int32, device=DEV)
    out.ext_nall = torch.empty((len(frames),), dtype=torch.int32, device=DEV)
    tol = dict(atol=1e-12, rtol=1e-12) if dtype == torch.float64 else dict(atol=5e-6, rtol=5e-6)
    dtol = dict(atol=1e-10, rtol=1e-10) if dtype == torch.float64 else dict(atol=2e-5, rtol=2e-5)
    plan = gb.NeighborPlan(nl, boxes, 6.0, DEV, dtype)
    npd = np.float64 if dtype == torch.float64 else np.float32
    for step, c in enumerate([c0, _displace(c0, 1), _displace(c0, 2)]):
        ct = torch.tensor(c, dtype=dtype, device=DEV)
        ops.env_mat_skin(skin_plan, vl, ct, t, avg, std, 6.0, 0.5, SEL, rebuild=(step == 0),
                         out=out, check_status=True)
        torch.cuda.synchronize()
        # the reference's formatting of the extended coordinates the step
        # used (ghosts refreshed from their atoms): bit-exact
        for f in range(len(frames)):
            a0, n_f = int(skin_plan.atom_off[f]), nl[f]
            e0, ne = int(skin_plan.ext_off[f]), int(out.ext_nall[f])
            ec = out.ext_coord[e0:e0 + ne].cpu().numpy().astype(npd)
            et = out.ext_type[e0:e0 + ne].cpu().numpy()
            ref = oracle.format_nlist(ec, et, n_f, 6.0, SEL)
            np.testing.assert_array_equal(out.nlist_ext[a0:a0 + n_f].cpu().numpy(), ref)
        if dtype == torch.float64:
            # and a fresh build at the same coordinates (its ghosts round the
            # same within 1e-15 A: no near-tie can swap)
            fresh = gb.env_mat_packed(plan, ct, t, avg, std, 0.5, SEL)
            torch.cuda.synchronize()
            assert torch.equal(out.nlist, fresh.nlist), step
            torch.testing.assert_close(out.em, fresh.em, **tol)
            torch.testing.assert_close(out.em_deriv, fresh.em_deriv, **dtol)
            torch.testing.assert_close(out.rij, fresh.rij, **tol)


def test_fused_step_on_reused_list(gb, mods):
    se_a, mdl, water, ops = mods
    cfg = mdl.SeAConfig()
    m = se_a.build_model(cfg, 17, [water.water_frame(4, 12.42, 1000)], DEV, torch.float64)
    frames = _frames(water)
    at = [f[1] for f in frames]
    boxes = np.stack([f[2] for f in frames])
    c0 = np.concatenate([f[0] for f in frames])
    c1 = _displace(c0, 5)
    bs = m.batch(at, boxes, skin=2.0)
    bf = m.batch(at, boxes)
    m.step_fused(bs, torch.tensor(c0, device=DEV), rebuild=True)
    Es, Fs, Vs = [x.clone() for x in m.step_fused(bs, torch.tensor(c1, device=DEV), rebuild=False)]
    Ef, Ff, Vf = m.step_fused(bf, torch.tensor(c1, device=DEV))
    torch.cuda.synchronize()
    assert bs.status() == 0
    assert float((Es - Ef).abs().max()) <= 1e-10 * len(c0)
    assert float((Fs - Ff).abs().max()) <= 1e-9
    assert float((Vs - Vf).abs().max()) <= 1e-8


def test_nve_with_skin_follows_rebuild_every_step(gb, mods):
    se_a, mdl, water, ops = mods
    md = importlib.import_module("dpmd_public_gb300.md")
    cfg = mdl.SeAConfig()
    m64 = se_a.build_model(cfg, 17, [water.water_frame(4, 12.42, 1000)], DEV, torch.float64)
    import copy

    params = copy.deepcopy(m64.params_np)
    for net in params["fit"]:
        net["final"]["w"] = net["final"]["w"] * 0.01
        net["final"]["b"] = net["final"]["b"] * 0.01
    m = se_a.SeAModel(cfg, params, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), DEV,
                      torch.float64, m64.tables_np, m64.infos_np)
    c, t, b = water.water_frame(4, 12.42, 1001)
    v = md.maxwell_boltzmann(t, 330.0, 3)
    runs = []
    for skin in (0.0, 2.0):
        bt = m.batch([t], b[None], skin=skin)
        nve = md.NVE(m, bt, c, v, t, dt=0.5, rebuild_every=10)
        nve.capture()
        e0 = nve.total_energy()
        nve.run(35)
        torch.cuda.synchronize()
        assert bt.status() == 0
        runs.append((nve.x.cpu().numpy(), nve.total_energy() - e0))
    assert np.abs(runs[0][0] - runs[1][0]).max() <= 1e-8
    assert abs(runs[0][1] - runs[1][1]) <= 1e-8
