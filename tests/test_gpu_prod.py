"""GPU parity of prod_force_se_a / prod_virial_se_a (atomic and deterministic
scatter) and of their backward kernels, against the CPU oracle and the
reference's golden vectors.  Deterministic mode must also be bitwise
reproducible run to run."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _ops(gb):
    gb.load_library()


def _env(oracle, fx):
    posi = np.array(fx["posi"])
    atype = np.array(fx["atype"], np.int32)
    sec = fx["sec_a"]
    sel = [sec[i + 1] - sec[i] for i in range(len(sec) - 1)]
    ec, et, emap = oracle.copy_coord(posi, atype, np.array(fx["box"]), fx["rc"])
    nloc, nnei = len(atype), sum(sel)
    em, emd, rij, nl = oracle.prod_env_mat_a_ext(ec, et, nloc, np.zeros((2, nnei * 4)),
                                                 np.ones((2, nnei * 4)), fx["rc"], fx["rc_smth"], sel)
    return nloc, len(et), nnei, emd, rij, nl


@pytest.mark.parametrize("det", [False, True])
def test_golden_force_virial(gb, oracle, golden_lib, det):
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    fx = golden_lib["TestProdForceA"]
    nloc, nall, nnei, emd, rij, nl = _env(oracle, fx)
    net = 10 - np.arange(nloc * nnei * 4) * 0.01
    natoms = torch.tensor([nloc, nall, 2, 4], dtype=torch.int32)
    T = lambda a: torch.tensor(np.tile(a, (2, 1)) if a.ndim == 1 else a, device=DEV)
    f = ops.prod_force_se_a_impl(T(net), T(emd), T(nl.astype(np.int32)), natoms, nnei, 0, det)
    exp = np.array(fx["expected_force"])
    np.testing.assert_allclose(f.cpu().numpy(), np.tile(exp, (2, 1)), atol=1e-5)
    fv = golden_lib["TestProdVirialA"]
    v, av = ops.prod_virial_se_a_impl(T(net), T(emd), T(rij), T(nl.astype(np.int32)), natoms, nnei, 0, det)
    np.testing.assert_allclose(v[0].cpu().numpy(), fv["expected_virial"], atol=1e-5)
    np.testing.assert_allclose(av[0].cpu().numpy(), fv["expected_atom_virial"], atol=1e-5)


def test_golden_grads(gb, oracle, golden_lib):
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    fx = golden_lib["TestProdForceGradA"]
    nloc, nall, nnei, emd, rij, nl = _env(oracle, fx)
    grad = 10 - np.arange(nloc * 3) * 0.1
    T = lambda a: torch.tensor(a, device=DEV)
    g = ops.prod_force_grad_impl(T(np.tile(grad, 2)), T(np.tile(emd, 2)), T(np.tile(nl, 2).astype(np.int32)),
                                 nloc, nnei, 2)
    np.testing.assert_allclose(g.cpu().numpy().reshape(-1), np.tile(fx["expected_grad_net"], 2), atol=1e-5)
    fv = golden_lib["TestProdVirialGradA"]
    gv = ops.prod_virial_grad_impl(T(10 - np.arange(9) * 1.0), T(emd), T(rij), T(nl.astype(np.int32)),
                                   nloc, nnei, 1)
    np.testing.assert_allclose(gv.cpu().numpy().reshape(-1), fv["expected_grad_net"], atol=1e-5)


def _water_case(gb, oracle, dtype, n=4, L=12.42, seed=4):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    c, t, b = water.water_frame(n, L, seed)
    sel = [46, 92]
    nnei = sum(sel)
    npd = np.float64 if dtype == torch.float64 else np.float32
    avg = np.zeros((2, nnei * 4), npd)
    std = np.ones((2, nnei * 4), npd)
    em, emd, rij, nl = oracle.prod_env_mat_a_pbc(c.astype(npd), t, b.astype(npd), avg, std, 6.0, 0.5, sel)
    rng = np.random.default_rng(seed)
    net = rng.normal(0, 1, em.shape).astype(npd)
    return len(t), nnei, net, emd, rij, nl


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("det", [False, True])
def test_water_vs_oracle(gb, oracle, dtype, det):
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    nloc, nnei, net, emd, rij, nl = _water_case(gb, oracle, dtype)
    natoms = torch.tensor([nloc, nloc, 0, 0], dtype=torch.int32)
    T = lambda a: torch.tensor(a.reshape(1, -1), device=DEV)
    f = ops.prod_force_se_a_impl(T(net), T(emd), T(nl), natoms, nnei, 0, det)
    v, av = ops.prod_virial_se_a_impl(T(net), T(emd), T(rij), T(nl), natoms, nnei, 0, det)
    fo = oracle.prod_force_a(net, emd, nl, nloc, nloc, nnei)
    vo, avo = oracle.prod_virial_a(net, emd, rij, nl, nloc, nloc, nnei)
    tol = dict(atol=1e-10, rtol=1e-10) if dtype == torch.float64 else dict(atol=2e-3, rtol=1e-4)
    np.testing.assert_allclose(f.cpu().numpy(), fo, **tol)
    np.testing.assert_allclose(av.cpu().numpy().reshape(-1), avo, **tol)
    vtol = dict(atol=1e-9, rtol=1e-10) if dtype == torch.float64 else dict(atol=5e-2, rtol=1e-4)
    np.testing.assert_allclose(v.cpu().numpy().reshape(-1), vo, **vtol)


def test_deterministic_is_bitwise_reproducible(gb, oracle):
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    nloc, nnei, net, emd, rij, nl = _water_case(gb, oracle, torch.float32, n=8, L=24.84, seed=6)
    natoms = torch.tensor([nloc, nloc, 0, 0], dtype=torch.int32)
    T = lambda a: torch.tensor(a.reshape(1, -1), device=DEV)
    runs = [ops.prod_force_se_a_impl(T(net), T(emd), T(nl), natoms, nnei, 0, True) for _ in range(3)]
    vir = [ops.prod_virial_se_a_impl(T(net), T(emd), T(rij), T(nl), natoms, nnei, 0, True)[0] for _ in range(3)]
    for a in runs[1:]:
        assert torch.equal(a, runs[0])
    for a in vir[1:]:
        assert torch.equal(a, vir[0])


def test_force_autograd_second_order(gb, oracle):
    """torch.ops.deepmd.prod_force_se_a is differentiable wrt net_deriv
    (prod_force_grad), as a force-loss training step needs."""
    nloc, nnei, net, emd, rij, nl = _water_case(gb, oracle, torch.float64, n=2, L=6.2, seed=9)
    natoms = torch.tensor([nloc, nloc, 0, 0], dtype=torch.int32)
    netT = torch.tensor(net.reshape(1, -1), device=DEV, requires_grad=True)
    f = torch.ops.deepmd.prod_force_se_a(netT, torch.tensor(emd.reshape(1, -1), device=DEV),
                                         torch.tensor(nl.reshape(1, -1), device=DEV), natoms, nnei, 0)
    w = torch.linspace(-1, 1, f.numel(), dtype=f.dtype, device=DEV).reshape(f.shape)
    (f * w).sum().backward()
    go = oracle.prod_force_grad_a(w.cpu().numpy().reshape(-1), emd, nl, nloc, nnei)
    np.testing.assert_allclose(netT.grad.cpu().numpy().reshape(-1), go, atol=1e-10)


@pytest.mark.parametrize("det", [False, True])
def test_many_frames_virial(gb, oracle, det):
    """40 frames in one call (9 x 40 = 360 virial words, more than one
    256-thread block): every frame's virial and atom virial against the
    oracle, nothing left at a zero fill."""
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    nloc, nnei, net, emd, rij, nl = _water_case(gb, oracle, torch.float64, n=2, L=6.2, seed=21)
    nf = 40
    rng = np.random.default_rng(3)
    nets = rng.normal(0, 1, (nf, net.size))
    natoms = torch.tensor([nloc, nloc, 0, 0], dtype=torch.int32)
    rep = lambda a: torch.tensor(np.tile(a.reshape(1, -1), (nf, 1)), device=DEV)
    v, av = ops.prod_virial_se_a_impl(torch.tensor(nets, device=DEV), rep(emd), rep(rij), rep(nl),
                                      natoms, nnei, 0, det)
    f = ops.prod_force_se_a_impl(torch.tensor(nets, device=DEV), rep(emd), rep(nl), natoms, nnei,
                                 0, det)
    for k in (0, 17, nf - 1):
        vo, avo = oracle.prod_virial_a(nets[k], emd, rij, nl, nloc, nloc, nnei)
        fo = oracle.prod_force_a(nets[k], emd, nl, nloc, nloc, nnei)
        np.testing.assert_allclose(v[k].cpu().numpy(), np.reshape(vo, -1), atol=1e-9, rtol=1e-10)
        np.testing.assert_allclose(av[k].cpu().numpy(), np.reshape(avo, -1), atol=1e-10, rtol=1e-10)
        np.testing.assert_allclose(f[k].cpu().numpy(), np.reshape(fo, -1), atol=1e-10, rtol=1e-10)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("det", [0, 1])
def test_force_virial_in_one_pass(gb, oracle, dtype, det):
    """gbdp_prod_force_virial_a_* equals the two separate ops: bit for bit in
    the deterministic mode, within floating-point atomics order otherwise."""
    import importlib

    ops = importlib.import_module("dpmd_public_gb300.ops")
    water = importlib.import_module("dpmd_public_gb300.water")
    frames = [water.water_frame(4, 12.42, 81), water.water_frame(4, 12.42, 82)]
    nnei = 138
    npd = np.float64 if dtype == torch.float64 else np.float32
    avg = np.zeros((2, nnei * 4))
    std = np.ones((2, nnei * 4))
    ems, emds, rijs, nls = [], [], [], []
    for c, t, b in frames:
        em, emd, rij, nl = oracle.prod_env_mat_a_pbc(c.astype(npd), t, b.astype(npd),
                                                     avg.astype(npd), std.astype(npd), 6.0, 0.5,
                                                     [46, 92])
        ems.append(em), emds.append(emd), rijs.append(rij), nls.append(nl)
    n = len(frames[0][1])
    rng = np.random.default_rng(83)
    net = torch.tensor(rng.normal(0, 1, (2, n * nnei * 4)), dtype=dtype, device="cuda")
    ed = torch.tensor(np.stack(emds), dtype=dtype, device="cuda")
    rij = torch.tensor(np.stack(rijs), dtype=dtype, device="cuda")
    nl = torch.tensor(np.stack(nls), dtype=torch.int32, device="cuda")
    natoms = torch.tensor([n, n, 0, 0], dtype=torch.int32)
    f1 = ops.prod_force_se_a_impl(net, ed, nl, natoms, nnei, 0, bool(det))
    v1, av1 = ops.prod_virial_se_a_impl(net, ed, rij, nl, natoms, nnei, 0, bool(det))
    f2, v2, av2 = ops.prod_force_virial_se_a_impl(net, ed, rij, nl, natoms, nnei, 0, bool(det))
    torch.cuda.synchronize()
    if det:
        assert torch.equal(f1, f2) and torch.equal(v1, v2) and torch.equal(av1, av2)
    else:
        tol = 1e-12 if dtype == torch.float64 else 2e-5
        for a, b in ((f1, f2), (v1, v2), (av1, av2)):
            assert float((a - b).abs().max()) <= tol * max(1.0, float(a.abs().max()))


def test_many_frames_force_fp32(gb, oracle):
    """FP32 atomic force over 40 frames in one call: the forces accumulate
    in padded 16-byte rows of the workspace (frame f, atom j at row
    f * nall + j) and are compacted into [nframes, nall * 3]; every frame
    against the oracle, nothing left at a zero fill."""
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    nloc, nnei, net, emd, rij, nl = _water_case(gb, oracle, torch.float32, n=2, L=6.2, seed=29)
    nf = 40
    nets = np.random.default_rng(8).normal(0, 1, (nf, net.size)).astype(np.float32)
    natoms = torch.tensor([nloc, nloc, 0, 0], dtype=torch.int32)
    rep = lambda a: torch.tensor(np.tile(a.reshape(1, -1), (nf, 1)), device=DEV)
    f = ops.prod_force_se_a_impl(torch.tensor(nets, device=DEV), rep(emd), rep(nl), natoms, nnei, 0)
    assert f.shape == (nf, nloc * 3)
    for k in range(nf):
        fo = oracle.prod_force_a(nets[k], emd, nl, nloc, nloc, nnei)
        np.testing.assert_allclose(f[k].cpu().numpy(), np.reshape(fo, -1), atol=2e-3, rtol=1e-4)
