"""GPU parity of torch.ops.deepmd.tabulate_fusion_se_a (forward, backward,
double backward) against the reference's golden vectors and the CPU oracle.
Tolerances: the reference PT test's (1e-10 fp64, 1e-5 fp32) on its golden
data; on random tables 1e-10 (fp64) and 2e-5 relative (fp32)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _ops(gb):
    gb.load_library()


def _pt_data(golden_pt, dtype):
    g = golden_pt
    t = lambda k, shape=None: torch.tensor(g[k]["values"], dtype=dtype)
    table = t("table_tensor").reshape(-1, 48).to(DEV)
    info = t("table_info_tensor")  # CPU, as the reference requires
    em_x = t("em_x_tensor").reshape(4, 4).to(DEV)
    em = t("em_tensor").reshape(4, 4, 4).to(DEV)
    return table, info, em_x, em


@pytest.mark.parametrize("dtype,prec", [(torch.float64, 1e-10), (torch.float32, 1e-5)])
def test_pt_golden_forward_backward(golden_pt, dtype, prec):
    table, info, em_x, em = _pt_data(golden_pt, dtype)
    em_x.requires_grad_(True)
    em.requires_grad_(True)
    out = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, 8)[0]
    exp = torch.tensor(golden_pt["expected_descriptor_tensor"]["values"], dtype=dtype).reshape(4, 4, 8)
    torch.testing.assert_close(out.cpu(), exp, atol=prec, rtol=prec)
    out.sum().backward()
    gx = torch.tensor(golden_pt["expected_dy_dem_x"]["values"], dtype=dtype).reshape(4, 4)
    gm = torch.tensor(golden_pt["expected_dy_dem"]["values"], dtype=dtype).reshape(4, 4, 4)
    torch.testing.assert_close(em_x.grad.cpu(), gx, atol=prec, rtol=prec)
    torch.testing.assert_close(em.grad.cpu(), gm, atol=prec, rtol=prec)


def test_lib_golden(golden_lib):
    fx = golden_lib["TestTabulateSeA"]
    nloc, nnei, M = fx["nloc"], fx["nnei"], fx["last_layer_size"]
    table = torch.tensor(fx["table"], dtype=torch.float64).reshape(-1, 6 * M).to(DEV)
    info = torch.tensor(fx["info"], dtype=torch.float64)
    em_x = torch.tensor(fx["em_x"], dtype=torch.float64).reshape(nloc, nnei).to(DEV).requires_grad_()
    em = torch.tensor(fx["em"], dtype=torch.float64).reshape(nloc, nnei, 4).to(DEV).requires_grad_()
    out = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, M)[0]
    np.testing.assert_allclose(out.detach().cpu().numpy().reshape(-1), fx["expected_xyz_scatter"], atol=1e-5)
    out.backward(torch.ones_like(out))
    np.testing.assert_allclose(em_x.grad.cpu().numpy().reshape(-1), fx["expected_dy_dem_x"], atol=1e-5)
    np.testing.assert_allclose(em.grad.cpu().numpy().reshape(-1), fx["expected_dy_dem"], atol=1e-5)


def _nonuniform(t):
    v = torch.linspace(-0.7, 1.3, t.numel(), dtype=t.dtype, device=t.device).reshape(t.shape)
    return v + 0.05 * torch.sin(torch.arange(t.numel(), dtype=t.dtype, device=t.device).reshape(t.shape))


def test_second_order_matches_finite_difference(golden_pt):
    """The reference PT test's grad-grad check (tabulate_test_utils.py:38-92):
    dz/dy from the grad-grad kernel vs central differences, fp64."""
    table, info, em_x, em = _pt_data(golden_pt, torch.float64)
    em_x.requires_grad_(True)
    em.requires_grad_(True)
    out = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, 8)[0]
    dy = _nonuniform(out).requires_grad_(True)
    g1 = torch.autograd.grad(out, (em_x, em), grad_outputs=dy, create_graph=True)
    w = tuple(_nonuniform(g) for g in g1)
    proj = sum((a * b).sum() for a, b in zip(g1, w))
    dz = torch.autograd.grad(proj, dy)[0]

    def project(dyv):
        o = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, 8)[0]
        gg = torch.autograd.grad(o, (em_x, em), grad_outputs=dyv)
        return sum((a * b).sum() for a, b in zip(gg, w))

    ref = torch.empty_like(dy)
    eps = 1e-6
    base = dy.detach()
    for k in range(dy.numel()):
        p, m = base.clone(), base.clone()
        p.view(-1)[k] += eps
        m.view(-1)[k] -= eps
        ref.view(-1)[k] = (project(p) - project(m)) / (2 * eps)
    torch.testing.assert_close(dz, ref, atol=1e-6, rtol=1e-6)


def _random_case(rng, dtype, nloc, nnei, M, pad=True):
    lower, upper, mx, s0, s1 = -1.0, 2.0, 10.0, 0.01, 0.1
    nrow = int((upper - lower) / s0) + int((mx - upper) / s1)
    table = rng.normal(0, 0.3, (nrow, 6 * M))
    info = np.array([lower, upper, mx, s0, s1, -1.0])
    em = rng.normal(0, 1, (nloc, nnei, 4))
    em_x = rng.uniform(-1.5, 11.0, (nloc, nnei))
    em_x[:, : nnei // 2] = rng.uniform(-0.9, 1.9, (nloc, nnei // 2))
    if pad:
        for i in range(nloc):
            k = rng.integers(0, nnei + 1)
            if k < nnei:
                em[i, k:, 1:] = 0.0
                em[i, k:, 0] = -0.6
                em_x[i, k:] = -0.6
    return table, info, em_x, em


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("nloc,nnei,M", [(97, 46, 100), (64, 92, 100), (5, 7, 33),
                                         (9, 40, 200), (3, 1, 8)])
def test_random_vs_oracle(oracle, dtype, nloc, nnei, M):
    rng = np.random.default_rng(nloc * 1000 + nnei + M)
    table, info, em_x, em = _random_case(rng, dtype, nloc, nnei, M)
    npd = np.float64 if dtype == torch.float64 else np.float32
    table, em_x, em, info_n = (a.astype(npd) for a in (table, em_x, em, info))
    T = lambda a: torch.tensor(a, device=DEV)
    tol = dict(atol=1e-10, rtol=1e-10) if dtype == torch.float64 else dict(atol=2e-5, rtol=2e-5)
    ex = T(em_x).requires_grad_()
    emt = T(em).requires_grad_()
    out = torch.ops.deepmd.tabulate_fusion_se_a(T(table), torch.tensor(info_n), ex, emt, M)[0]
    ref = oracle.tabulate_fusion_se_a(table, info_n, em_x.reshape(-1, 1), em, M)
    scale = max(1.0, float(np.abs(ref).max()))
    np.testing.assert_allclose(out.detach().cpu().numpy() / scale, ref / scale, **tol)
    dy = rng.normal(0, 1, (nloc, 4, M)).astype(npd)
    out.backward(T(dy))
    gx, gm = oracle.tabulate_fusion_se_a_grad(table, info_n, em_x.reshape(-1, 1), em, dy)
    sx = max(1.0, float(np.abs(gx).max()))
    sm = max(1.0, float(np.abs(gm).max()))
    np.testing.assert_allclose(ex.grad.cpu().numpy() / sx, gx.reshape(nloc, nnei) / sx, **tol)
    np.testing.assert_allclose(emt.grad.cpu().numpy() / sm, gm / sm, **tol)
    # grad-grad through the internal op
    dzx = rng.normal(0, 1, (nloc, nnei)).astype(npd)
    dzm = rng.normal(0, 1, (nloc, nnei, 4)).astype(npd)
    ops = __import__("dpmd_public_gb300.ops", fromlist=["x"])
    dz = ops.tabulate_grad_grad(T(table), torch.tensor(info_n), T(em_x), T(em), T(dzx), T(dzm), M)
    dzo = oracle.tabulate_fusion_se_a_grad_grad(table, info_n, em_x.reshape(-1, 1), em, dzx, dzm, M)
    sz = max(1.0, float(np.abs(dzo).max()))
    np.testing.assert_allclose(dz.cpu().numpy() / sz, dzo / sz, **tol)


def test_empty_inputs():
    table = torch.zeros(10, 48, dtype=torch.float64, device=DEV)
    info = torch.tensor([0, 0.05, 0.1, 0.01, 0.01, -1], dtype=torch.float64)
    out = torch.ops.deepmd.tabulate_fusion_se_a(
        table, info, torch.zeros(0, 4, dtype=torch.float64, device=DEV),
        torch.zeros(0, 4, 4, dtype=torch.float64, device=DEV), 8)[0]
    assert out.shape == (0, 4, 8)


def test_cpu_tensors_fail_loudly():
    table = torch.zeros(10, 48, dtype=torch.float64)
    info = torch.tensor([0, 0.05, 0.1, 0.01, 0.01, -1], dtype=torch.float64)
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        torch.ops.deepmd.tabulate_fusion_se_a(table, info, torch.zeros(2, 4, dtype=torch.float64),
                                              torch.zeros(2, 4, 4, dtype=torch.float64), 8)


@pytest.mark.parametrize("dtype,m", [(torch.float32, 100), (torch.float32, 37), (torch.float64, 100),
                                     (torch.float64, 16)])
def test_table_to_planar_layout(gb, dtype, m):
    """gbdp_table_to_planar_*: element (r, 2p + c, k) of the [nrow, 6 M]
    coefficient-minor table lands at r * row_elems + p * P + 2 k + c, with
    zero padding up to the plane pitch P (2 M rounded up to 128 bytes)."""
    import ctypes

    L = gb._lib
    lib = L.load()
    nrow = 7
    rng = np.random.default_rng(3)
    src_np = rng.standard_normal((nrow, 6 * m))
    src = torch.tensor(src_np, dtype=dtype, device=DEV)
    esz = src.element_size()
    re = lib.gbdp_table_planar_row_elems(m, esz)
    pitch = re // 3
    assert pitch * esz % 128 == 0 and pitch >= 2 * m
    dst = torch.full((nrow * re,), 7.0, dtype=dtype, device=DEV)
    fn = lib.gbdp_table_to_planar_f64 if dtype == torch.float64 else lib.gbdp_table_to_planar_f32
    L.check(fn(dst.data_ptr(), src.data_ptr(), nrow, m, None), "table_to_planar")
    torch.cuda.synchronize()
    got = dst.cpu().numpy().reshape(nrow, 3, pitch)
    exp = np.zeros((nrow, 3, pitch))
    co = src_np.reshape(nrow, m, 3, 2)  # [r, k, p, c]
    exp[:, :, :2 * m] = co.transpose(0, 2, 1, 3).reshape(nrow, 3, 2 * m)
    np.testing.assert_array_equal(got, exp.astype(got.dtype))
