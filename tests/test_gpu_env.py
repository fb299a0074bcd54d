"""GPU parity of the periodic neighbour build + environment matrix.

The neighbour list (order inside each type section, padding, mapping back to
local atoms) must be bit-exact against the reference; env values within
1e-12 (fp64) / 5e-6 (fp32, derivative rows 2e-5 absolute); em is compared
with the reference library's own output (golden fixture)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
SEL = [46, 92]
NNEI = sum(SEL)


@pytest.fixture(scope="module", autouse=True)
def _ops(gb):
    gb.load_library()


def _run(gb, coords, types, boxes, avg, std, dtype, rcut=6.0, rcut_smth=0.5, sel=SEL,
         max_cand=0):
    plan = gb.NeighborPlan([len(t) for t in types], np.stack([np.asarray(b).reshape(9) for b in boxes]),
                           rcut, DEV, dtype, max_cand=max_cand)
    c = torch.tensor(np.concatenate(coords), dtype=dtype, device=DEV)
    t = torch.tensor(np.concatenate(types), dtype=torch.int32, device=DEV)
    r = gb.env_mat_packed(plan, c, t, torch.tensor(avg, dtype=dtype, device=DEV),
                          torch.tensor(std, dtype=dtype, device=DEV), rcut_smth, sel,
                          need_nlist_ext=True)
    return plan, r


def _stats(dtype, seed=0, sel=SEL):
    rng = np.random.default_rng(seed)
    nn = sum(sel)
    avg = np.zeros((len(sel), nn * 4))
    avg[:, 0::4] = rng.uniform(0.05, 0.15, (len(sel), nn))
    std = np.ones((len(sel), nn * 4))
    std[:, 0::4] = rng.uniform(0.1, 0.2, (len(sel), nn))
    std[:, 1::4] = std[:, 2::4] = std[:, 3::4] = rng.uniform(0.05, 0.1, (len(sel), nn))
    return avg, std


@pytest.mark.parametrize("tag", ["w192", "w24", "w1536"])
@pytest.mark.parametrize("sfx,dtype", [("f64", torch.float64), ("f32", torch.float32)])
def test_vs_reference_fixture(gb, golden_water, tag, sfx, dtype):
    g = golden_water
    npd = np.float64 if dtype == torch.float64 else np.float32
    c, t, b = g[f"{tag}_coord"].astype(npd), g[f"{tag}_atype"], g[f"{tag}_box"]
    plan, r = _run(gb, [c], [t], [b], g["avg"], g["std"], dtype)
    nl = r.nlist.cpu().numpy().reshape(-1)
    np.testing.assert_array_equal(nl, g[f"{tag}_{sfx}_nlist"].astype(np.int32))
    assert int(r.ext_nall[0]) == int(g[f"{tag}_{sfx}_nall"])
    n = int(g[f"{tag}_{sfx}_nall"])
    np.testing.assert_array_equal(r.ext_map[:n].cpu().numpy(), g[f"{tag}_{sfx}_mapping"].astype(np.int32))
    keep = 24 * NNEI
    tol = dict(atol=1e-12, rtol=1e-12) if dtype == torch.float64 else dict(atol=5e-6, rtol=5e-6)
    # fp32 derivative rows: terms of size ~1/r^2 cancel, so the bound is
    # absolute (2e-5) rather than relative to each component
    dtol = dict(atol=1e-12, rtol=1e-12) if dtype == torch.float64 else dict(atol=2e-5, rtol=2e-5)
    np.testing.assert_allclose(r.em.cpu().numpy().reshape(-1)[: keep * 4], g[f"{tag}_{sfx}_em"], **tol)
    np.testing.assert_allclose(r.em_deriv.cpu().numpy().reshape(-1)[: keep * 12],
                               g[f"{tag}_{sfx}_em_deriv"], **dtol)
    np.testing.assert_allclose(r.rij.cpu().numpy().reshape(-1)[: keep * 3], g[f"{tag}_{sfx}_rij"], **tol)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_ragged_batch_vs_oracle(gb, oracle, dtype):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    frames = water.ragged_frames(7, seed=3, lo=8, hi=200)
    frames.append(water.water_frame(2, 6.2, 99))  # single-cell box, 26 ghost images
    npd = np.float64 if dtype == torch.float64 else np.float32
    avg, std = _stats(dtype, 1)
    coords = [f[0].astype(npd) for f in frames]
    plan, r = _run(gb, coords, [f[1] for f in frames], [f[2] for f in frames], avg, std, dtype)
    off = 0
    for k, (c, t, b) in enumerate(frames):
        n = len(t)
        em, emd, rij, nl, ec, et, emap = oracle.prod_env_mat_a_pbc(
            c.astype(npd), t, b.astype(npd), avg.astype(npd), std.astype(npd), 6.0, 0.5, SEL,
            return_ext=True)
        np.testing.assert_array_equal(r.nlist[off:off + n].cpu().numpy().reshape(-1), nl)
        assert int(r.ext_nall[k]) == len(et)
        eo = int(plan.ext_off[k])
        np.testing.assert_array_equal(r.ext_coord[eo:eo + len(et)].cpu().numpy(), ec)
        np.testing.assert_array_equal(r.ext_map[eo:eo + len(et)].cpu().numpy(), emap)
        tol = dict(atol=1e-12, rtol=1e-12) if dtype == torch.float64 else dict(atol=5e-6, rtol=5e-6)
        dtol = dict(atol=1e-12, rtol=1e-12) if dtype == torch.float64 else dict(atol=2e-5, rtol=2e-5)
        np.testing.assert_allclose(r.em[off:off + n].cpu().numpy().reshape(-1), em, **tol)
        np.testing.assert_allclose(r.em_deriv[off:off + n].cpu().numpy().reshape(-1), emd, **dtol)
        off += n


@pytest.mark.parametrize("name", ["TestEnvMatA", "TestEnvMatAShortSel"])
def test_lib_golden_env(gb, golden_lib, name):
    """The reference's 6-atom fixture (13 A box, rc 6, rc_smth 0.8) with
    avg 0 / std 1: the golden env values of test_env_mat_a.cc."""
    fx = golden_lib[name]
    sec = fx["sec_a"]
    sel = [sec[i + 1] - sec[i] for i in range(len(sec) - 1)]
    nn = sum(sel)
    avg = np.zeros((2, nn * 4))
    std = np.ones((2, nn * 4))
    c = np.array(fx["posi"]).reshape(-1, 3)
    t = np.array(fx["atype"], np.int32)
    plan, r = _run(gb, [c], [t], [np.array(fx["box"])], avg, std, torch.float64, rcut=fx["rc"],
                   rcut_smth=fx["rc_smth"], sel=sel)
    np.testing.assert_allclose(r.em.cpu().numpy().reshape(-1), fx["expected_env"], atol=1e-5)


@pytest.mark.parametrize("name", ["TestFormatNlist", "TestFormatNlistShortSel"])
def test_lib_golden_format_nlist(gb, golden_lib, name):
    """test_fmt_nlist.cc golden lists, in the extended (copy_coord) index space."""
    fx = golden_lib[name]
    sec = fx["sec_a"]
    sel = [sec[i + 1] - sec[i] for i in range(len(sec) - 1)]
    nn = sum(sel)
    c = np.array(fx["posi"]).reshape(-1, 3)
    t = np.array(fx["atype"], np.int32)
    plan, r = _run(gb, [c], [t], [np.array(fx["box"])], np.zeros((2, nn * 4)), np.ones((2, nn * 4)),
                   torch.float64, rcut=fx["rc"], sel=sel)
    np.testing.assert_array_equal(r.nlist_ext.cpu().numpy().reshape(-1), fx["expect_nlist_cpy"])


def test_tf_contract_op_multi_frame(gb, oracle):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    fr = [water.water_frame(4, 12.42, s) for s in (21, 22, 23)]
    c = np.stack([f[0].reshape(-1) for f in fr])
    t = np.stack([f[1] for f in fr]).astype(np.int32)
    b = np.stack([f[2] for f in fr])
    avg, std = _stats(torch.float64, 5)
    natoms = torch.tensor([192, 192, 64, 128], dtype=torch.int32)
    mesh = torch.zeros(6, dtype=torch.int32)
    out = torch.ops.deepmd.prod_env_mat_a(
        torch.tensor(c, device=DEV), torch.tensor(t, device=DEV), natoms, torch.tensor(b, device=DEV),
        mesh, torch.tensor(avg, device=DEV), torch.tensor(std, device=DEV), 6.0, 6.0, 0.5, SEL, [0, 0])
    assert out[0].shape == (3, 192 * NNEI * 4) and out[3].dtype == torch.int32
    for k in range(3):
        em, emd, rij, nl = oracle.prod_env_mat_a_pbc(fr[k][0], fr[k][1], fr[k][2], avg, std, 6.0, 0.5, SEL)
        np.testing.assert_array_equal(out[3][k].cpu().numpy(), nl)
        np.testing.assert_allclose(out[0][k].cpu().numpy(), em, atol=1e-12)
        np.testing.assert_allclose(out[1][k].cpu().numpy(), emd, atol=1e-12)
        np.testing.assert_allclose(out[2][k].cpu().numpy(), rij, atol=1e-12)


def test_candidate_overflow_is_reported_and_retried(gb, oracle):
    """A max_cand smaller than the real neighbour count raises the device
    status word (no fault, no hang); the host wrapper doubles the capacity
    until every centre's candidates fit (16 -> 128 for water, about 90
    within rc) and returns the reference's list."""
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    c, t, b = water.water_frame(4, 12.42, 2)
    avg, std = _stats(torch.float64, 2)
    plan, r = _run(gb, [c], [t], [b], avg, std, torch.float64, max_cand=16)
    assert plan.max_cand == 128
    em, emd, rij, nl = oracle.prod_env_mat_a_pbc(c, t, b, avg, std, 6.0, 0.5, SEL)
    np.testing.assert_array_equal(r.nlist.cpu().numpy().reshape(-1), nl)


def test_sel_overflow_keeps_nearest(gb, oracle):
    """Short sel: the farthest neighbours of each type are dropped exactly
    as format_nlist_i_cpu drops them."""
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    c, t, b = water.water_frame(4, 12.42, 8)
    sel = [10, 20]
    nn = 30
    avg = np.zeros((2, nn * 4))
    std = np.ones((2, nn * 4))
    plan, r = _run(gb, [c], [t], [b], avg, std, torch.float64, sel=sel)
    em, emd, rij, nl = oracle.prod_env_mat_a_pbc(c, t, b, avg, std, 6.0, 0.5, sel)
    np.testing.assert_array_equal(r.nlist.cpu().numpy().reshape(-1), nl)


# ------------------------------------------------- forward_lower (external nlist) --
def _golden_pt_nlist():
    import os

    return np.load(os.path.join(os.path.dirname(__file__), "golden", "pt_format_nlist.npz"))


@pytest.mark.parametrize("sfx,dtype", [("f64", torch.float64), ("f32", torch.float32)])
def test_external_nlist_vs_reference_pt_formatting(gb, oracle, sfx, dtype):
    """prod_env_mat_a_nlist on an unsorted rcut + skin candidate list: the
    formatted list equals the reference's own PyTorch formatting (golden
    fixture) bit for bit; env values match the oracle's env rows for that
    list within 1e-12 (fp64) / 5e-6 (fp32, derivative rows 2e-5)."""
    g = _golden_pt_nlist()
    nloc = int(g["nloc"])
    sel = [int(s) for s in g["sel"]]
    rcut = float(g["rcut"])
    npd = np.float64 if dtype == torch.float64 else np.float32
    avg, std = _stats(npd, seed=3, sel=sel)
    ext = g["ext_coord"].astype(npd)
    em, emd, rij, nl = torch.ops.deepmd.prod_env_mat_a_nlist(
        torch.tensor(ext[None], device=DEV), torch.tensor(g["ext_type"][None], device=DEV),
        torch.tensor(g["nlist_in"][None], device=DEV), torch.tensor(avg, device=DEV),
        torch.tensor(std, device=DEV), rcut, 0.5, sel)
    nl = nl.cpu().numpy().reshape(nloc, -1)
    np.testing.assert_array_equal(nl, g[f"{sfx}_nlist"])
    e_o, d_o, r_o = oracle.env_mat_a_nlist(ext, g["ext_type"], nl, nloc, avg, std, rcut, 0.5, sel)
    tol, dtol = (1e-12, 1e-12) if dtype == torch.float64 else (5e-6, 2e-5)
    np.testing.assert_allclose(em.cpu().numpy().reshape(-1), e_o, rtol=tol, atol=tol)
    np.testing.assert_allclose(emd.cpu().numpy().reshape(-1), d_o, rtol=dtol, atol=dtol)
    np.testing.assert_allclose(rij.cpu().numpy().reshape(-1), r_o, rtol=tol, atol=tol)


def test_external_nlist_multi_frame_vs_oracle(gb, oracle):
    """Two frames with differently shuffled lists, -1 padding interleaved
    and a list shorter than sum(sel) for some atoms; per frame the oracle's
    restatement of the forward_lower formatting gives the same list."""
    g = _golden_pt_nlist()
    nloc = int(g["nloc"])
    sel = [int(s) for s in g["sel"]]
    ext = g["ext_coord"]
    rng = np.random.default_rng(77)
    lists = []
    for f in range(2):
        nl = g["nlist_in"].copy()
        for i in range(nloc):
            row = nl[i]
            if f == 1 and i % 5 == 0:
                row[rng.random(row.size) < 0.5] = -1  # thin the list out
            nl[i] = row[rng.permutation(row.size)]
        lists.append(nl)
    nl_in = np.stack(lists)
    exts = np.stack([ext, ext + 0.0])
    types = np.stack([g["ext_type"]] * 2)
    avg, std = _stats(np.float64, seed=4, sel=sel)
    _, _, _, nl = torch.ops.deepmd.prod_env_mat_a_nlist(
        torch.tensor(exts, device=DEV), torch.tensor(types, device=DEV),
        torch.tensor(nl_in, device=DEV), torch.tensor(avg, device=DEV),
        torch.tensor(std, device=DEV), float(g["rcut"]), 0.5, sel)
    nl = nl.cpu().numpy().reshape(2, nloc, -1)
    for f in range(2):
        exp = oracle.format_nlist_pt(exts[f], types[f], nl_in[f], nloc, float(g["rcut"]), sel)
        np.testing.assert_array_equal(nl[f], exp)


def test_external_nlist_bad_index_is_reported(gb):
    """A listed index >= nall is skipped by the kernel and reported through
    the status word (an error on the host), never dereferenced."""
    g = _golden_pt_nlist()
    nloc = int(g["nloc"])
    sel = [int(s) for s in g["sel"]]
    nl_in = g["nlist_in"].copy()
    nl_in[3, 0] = len(g["ext_type"]) + 5
    avg, std = _stats(np.float64, seed=5, sel=sel)
    with pytest.raises(Exception, match="status"):
        torch.ops.deepmd.prod_env_mat_a_nlist(
            torch.tensor(g["ext_coord"][None], device=DEV),
            torch.tensor(g["ext_type"][None], device=DEV), torch.tensor(nl_in[None], device=DEV),
            torch.tensor(avg, device=DEV), torch.tensor(std, device=DEV), float(g["rcut"]), 0.5,
            sel)
