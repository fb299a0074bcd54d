"""Neighbour-list bit-exactness at the sizes whose configurations demand it.

The canonical order (type, float32 r^2, extended index) of
source/lib/src/fmt_nlist.cc:14-26,98-143 is checked element by element
against the CPU oracle (itself pinned to the reference library compiled from
its sources) on:

* the whole 12,288-atom frame (4096 H2O, 49.68 A box), fp32 and fp64;
* unjittered lattices whose exact coordinates give exact float32 r^2 ties
  by the thousand, so the index tie-break decides the order, including a
  dense one whose sections overflow sel (which tied atom is kept at the
  truncation is decided by the index as well) and whose outermost shell
  lies exactly on rc (r^2 == rc^2: the candidate test is strict);
* a sample of the 512-frame ragged batch (every frame's list taken from the
  one packed launch over all 398,850 atoms), the largest frames included.

Each case prints the number of float32 r^2 ties it meets between adjacent
entries of a section (run pytest with -s to see them)."""

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


def _stats(nt=2, seed=0):
    rng = np.random.default_rng(seed)
    avg = np.zeros((nt, NNEI * 4))
    avg[:, 0::4] = rng.uniform(0.05, 0.15, (nt, NNEI))
    std = np.ones((nt, NNEI * 4))
    std[:, 0::4] = rng.uniform(0.1, 0.2, (nt, NNEI))
    std[:, 1::4] = std[:, 2::4] = std[:, 3::4] = rng.uniform(0.05, 0.1, (nt, NNEI))
    return avg, std


def _gpu_env(gb, frames, dtype, avg, std, sel=SEL):
    plan = gb.NeighborPlan([len(f[1]) for f in frames], np.stack([f[2] for f in frames]), 6.0, DEV,
                           dtype)
    npd = np.float64 if dtype == torch.float64 else np.float32
    c = torch.tensor(np.concatenate([f[0].astype(npd) for f in frames]), dtype=dtype, device=DEV)
    t = torch.tensor(np.concatenate([f[1] for f in frames]), dtype=torch.int32, device=DEV)
    r = gb.env_mat_packed(plan, c, t, torch.tensor(avg, dtype=dtype, device=DEV),
                          torch.tensor(std, dtype=dtype, device=DEV), 0.5, sel, need_nlist_ext=True)
    torch.cuda.synchronize()
    return plan, r


def count_ties(ext_coord, nlist_ext, sel):
    """Adjacent entries of a section whose float32 r^2 (diff = (float)x_j -
    (float)x_i, r^2 = dx dx + dy dy + dz dz, each operation rounded) are
    equal: the places where only the index orders the list."""
    ec = np.asarray(ext_coord, np.float32)
    nl = np.asarray(nlist_ext).reshape(-1, sum(sel))
    d = ec[np.maximum(nl, 0)] - ec[np.arange(len(nl))][:, None, :]
    r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    ties = 0
    s0 = 0
    for s in sel:
        a, b = slice(s0, s0 + s - 1), slice(s0 + 1, s0 + s)
        ok = (nl[:, a] >= 0) & (nl[:, b] >= 0)
        ties += int(((r2[:, a] == r2[:, b]) & ok).sum())
        s0 += s
    return ties


def _check_frame(oracle, r, plan, k, frame, dtype, avg, std, label):
    c, t, b = frame
    npd = np.float64 if dtype == torch.float64 else np.float32
    n = len(t)
    a0 = int(plan.atom_off[k])
    em, emd, rij, nl, ec, et, emap = oracle.prod_env_mat_a_pbc(
        c.astype(npd), t, b.astype(npd), avg.astype(npd), std.astype(npd), 6.0, 0.5, SEL,
        return_ext=True, cell_list=True)
    np.testing.assert_array_equal(r.nlist[a0:a0 + n].cpu().numpy().reshape(-1), nl)
    assert int(r.ext_nall[k]) == len(et)
    eo = int(plan.ext_off[k])
    np.testing.assert_array_equal(r.ext_map[eo:eo + len(et)].cpu().numpy(), emap)
    np.testing.assert_array_equal(r.ext_coord[eo:eo + len(et)].cpu().numpy(), ec)
    # nlist_ext holds indices into the frame's own extended atoms
    nl_ext = r.nlist_ext[a0:a0 + n].cpu().numpy()
    ties = count_ties(ec, nl_ext, SEL)
    tol = dict(atol=1e-12, rtol=1e-12) if dtype == torch.float64 else dict(atol=5e-6, rtol=5e-6)
    np.testing.assert_allclose(r.em[a0:a0 + n].cpu().numpy().reshape(-1), em, **tol)
    print(f"[nlist] {label}: {n} atoms, {int((nl >= 0).sum())} entries, {ties} float32 r^2 ties")
    return ties


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_water_12288_atoms_bit_exact(gb, oracle, dtype):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    frame = water.water_frame(16, 49.68, 20261203)
    avg, std = _stats()
    plan, r = _gpu_env(gb, [frame], dtype, avg, std)
    _check_frame(oracle, r, plan, 0, frame, dtype, avg, std, f"water 12288 {dtype}")


def _lattice(n, a, seed):
    """n^3 sites of spacing a (exact binary fractions) in an n a box, types
    drawn at random with one in three of type 0: no jitter, so float32 r^2
    of symmetric neighbours are exactly equal."""
    rng = np.random.default_rng(seed)
    g = np.arange(n) * a
    c = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    perm = rng.permutation(len(c))  # index order unrelated to geometry
    c = c[perm]
    t = (rng.random(len(c)) < 2 / 3).astype(np.int32)
    return c, t, np.diag([n * a] * 3).reshape(-1).astype(np.float64)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n,a", [(10, 2.5), (8, 1.5)])
def test_lattice_ties_resolved_by_index(gb, oracle, dtype, n, a):
    """Spacing 2.5 A: about 58 neighbours per atom, no truncation; spacing
    1.5 A: about 250 within rc, both sections truncated to sel, and the
    shell at 4 a = 6 A lies exactly on rc (excluded by r^2 < rc^2)."""
    frame = _lattice(n, a, seed=int(a * 10) + n)
    avg, std = _stats()
    plan, r = _gpu_env(gb, [frame], dtype, avg, std)
    ties = _check_frame(oracle, r, plan, 0, frame, dtype, avg, std, f"lattice {n}^3 a={a} {dtype}")
    assert ties > 1000


def test_ragged_512_frames_sampled_bit_exact(gb, oracle):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    frames = water.ragged_frames(512, seed=20261203, lo=8, hi=512)
    avg, std = _stats(seed=2)
    plan, r = _gpu_env(gb, frames, torch.float32, avg, std)
    sizes = np.array([len(f[1]) for f in frames])
    order = np.argsort(sizes, kind="stable")
    pick = sorted(set(order[np.linspace(0, len(order) - 1, 20).round().astype(int)].tolist()
                      + order[-4:].tolist()))
    ties = 0
    for k in pick:
        ties += _check_frame(oracle, r, plan, k, frames[k], torch.float32, avg, std,
                             f"ragged frame {k}")
    assert max(sizes[pick]) == 1536
    print(f"[nlist] ragged sample: {len(pick)} frames, {ties} ties")


def test_candidate_overflow_doubles_capacity_and_retries(gb, oracle):
    """A 1 A lattice has about 900 candidates within rc per centre, above
    the default capacity of 512: the env-mat call doubles the capacity,
    runs again and returns the reference's list (truncated to sel)."""
    frame = _lattice(10, 1.0, seed=5)
    avg, std = _stats()
    plan, r = _gpu_env(gb, [frame], torch.float64, avg, std)
    assert plan.max_cand == 1024
    _check_frame(oracle, r, plan, 0, frame, torch.float64, avg, std, "lattice 10^3 a=1.0 retry")


def test_candidate_overflow_at_the_limit_raises(gb):
    """At the capacity limit the overflow is reported, not truncated."""
    frame = _lattice(10, 1.0, seed=5)
    avg, std = _stats()
    plan = gb.NeighborPlan([1000], frame[2][None], 6.0, DEV, torch.float64, max_cand=512)
    plan.MAX_CAND_LIMIT = 512
    c = torch.tensor(frame[0], device=DEV)
    t = torch.tensor(frame[1], dtype=torch.int32, device=DEV)
    with pytest.raises(RuntimeError, match="candidate overflow"):
        gb.env_mat_packed(plan, c, t, torch.tensor(avg, device=DEV), torch.tensor(std, device=DEV),
                          0.5, SEL)


def test_captured_step_retries_after_overflow(gb):
    """The captured fused step on the dense lattice: the first call
    overflows, the step is captured again with twice the capacity, and its
    forces equal an eager step's with that capacity."""
    import importlib

    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")
    water = importlib.import_module("dpmd_public_gb300.water")
    cfg = mdl.SeAConfig()
    m64 = se_a.build_model(cfg, 7, [water.water_frame(4, 12.42, 1000)], DEV, torch.float64)
    m = se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), DEV,
                      torch.float32, m64.tables_np, m64.infos_np)
    c, t, b = _lattice(10, 1.0, seed=5)
    # move the lattice off its exact sites so that forces are not all zero
    c = c + np.random.default_rng(1).normal(0, 0.05, c.shape)
    bt = m.batch([t], b[None])
    step = se_a.CapturedStep(m, bt, coord=c.astype(np.float32))
    E, F, V = step(c.astype(np.float32))
    assert bt.plan.max_cand == 1024 and bt.status() == 0
    b2 = m.batch([t], b[None], max_cand=1024)
    E2, F2, V2 = m.step_fused(b2, torch.tensor(c, dtype=torch.float32, device=DEV))
    torch.cuda.synchronize()
    assert torch.equal(F, F2.cpu())
