"""libdeepmd_op_gb300.so: the libtorch registration of the deepmd operators
(what a C++ TorchScript host such as DeepPotPT loads in place of the
reference's libdeepmd_op_pt.so).  Each check runs in a fresh interpreter that
loads only the shim, so the Python-side registration plays no part."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "dpmd-public_gb300", "libdeepmd_op_gb300.so")


def _run(code: str) -> dict:
    # from a file: TorchScript compiles a function from its source
    import tempfile

    with tempfile.NamedTemporaryFile("w", suffix=".py", delete=False) as fh:
        fh.write(code)
    try:
        r = subprocess.run([sys.executable, fh.name], capture_output=True, text=True, cwd=ROOT,
                           timeout=600)
    finally:
        os.unlink(fh.name)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_shim_registers_reference_schema(gb):
    """The shim loads, owns deepmd::enable_mpi and registers
    tabulate_fusion_se_a with the reference's schema; a CPU tensor raises
    instead of falling back."""
    assert os.path.exists(SHIM), "libdeepmd_op_gb300.so not built (run __graft_entry__.build())"
    out = _run(f"""
import json, torch
torch.ops.load_library({SHIM!r})
op = torch.ops.deepmd.tabulate_fusion_se_a.default
err = ""
try:
    torch.ops.deepmd.tabulate_fusion_se_a(torch.zeros(4, 48), torch.zeros(6), torch.zeros(4, 1),
                                          torch.zeros(4, 1, 4), 8)
except RuntimeError as e:
    err = str(e)
print(json.dumps({{"schema": str(op._schema), "mpi": bool(torch.ops.deepmd.enable_mpi()),
                   "err": err}}))
""")
    # inferred from the C++ signature, as the reference's own registration
    # (m.def("tabulate_fusion_se_a", fn), tabulate_multi_device.cc:1550-1552) is
    assert out["schema"] == ("deepmd::tabulate_fusion_se_a(Tensor _0, Tensor _1, Tensor _2, "
                             "Tensor _3, int _4) -> Tensor[] _0")
    assert out["mpi"] is False
    assert "CUDA tensors only" in out["err"]


@pytest.mark.gpu
def test_shim_golden_and_torchscript(gb):
    """Through the shim only: forward and backward on the reference PyTorch
    test's golden vectors (1e-10 fp64 / 1e-5 fp32, the reference test's
    tolerances), the grad-of-grad as the adjoint of the (linear in dy) grad
    to 1e-12, and a TorchScript function calling the op by name."""
    gb.load_library()
    golden = os.path.join(ROOT, "tests", "golden", "pt_tabulate.json")
    out = _run(f"""
import json, torch
torch.ops.load_library({SHIM!r})
g = json.load(open({golden!r}))
res = {{}}
for dt, tol in ((torch.float64, 1e-10), (torch.float32, 1e-5)):
    t = lambda k: torch.tensor(g[k]["values"], dtype=dt)
    table = t("table_tensor").reshape(-1, 48).cuda()
    info = t("table_info_tensor")
    em_x = t("em_x_tensor").reshape(4, 4).cuda().requires_grad_(True)
    em = t("em_tensor").reshape(4, 4, 4).cuda().requires_grad_(True)
    out = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, 8)[0]
    exp = t("expected_descriptor_tensor").reshape(4, 4, 8)
    e1 = float((out.cpu() - exp).abs().max())
    out.sum().backward()
    e2 = float((em_x.grad.cpu() - t("expected_dy_dem_x").reshape(4, 4)).abs().max())
    e3 = float((em.grad.cpu() - t("expected_dy_dem").reshape(4, 4, 4)).abs().max())
    res[str(dt)] = [e1, e2, e3, tol]
# grad-of-grad: the grad is linear in dy, so for any u the grad-grad kernel's
# vector-Jacobian product must satisfy <u, grad(dy)> = <gradgrad(u), dy>
dt = torch.float64
t = lambda k: torch.tensor(g[k]["values"], dtype=dt)
table = t("table_tensor").reshape(-1, 48).cuda(); info = t("table_info_tensor")
em_x = t("em_x_tensor").reshape(4, 4).cuda().requires_grad_(True)
em = t("em_tensor").reshape(4, 4, 4).cuda().requires_grad_(True)
gen = torch.Generator().manual_seed(5)
dy = torch.randn(4, 4, 8, generator=gen, dtype=dt).cuda().requires_grad_(True)
o = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, 8)[0]
gx, gm = torch.autograd.grad(o, (em_x, em), grad_outputs=dy, create_graph=True)
ux = torch.randn(gx.shape, generator=gen, dtype=dt).cuda()
um = torch.randn(gm.shape, generator=gen, dtype=dt).cuda()
s = (ux * gx).sum() + (um * gm).sum()
dz, = torch.autograd.grad(s, dy)
res["gradgrad_rel"] = float(abs((dz * dy).sum() - s) / abs(s))
@torch.jit.script
def scripted(table: torch.Tensor, info: torch.Tensor, em_x: torch.Tensor, em: torch.Tensor):
    return torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x, em, 8)[0]
o2 = scripted(table, info, em_x.detach(), em.detach())
o1 = torch.ops.deepmd.tabulate_fusion_se_a(table, info, em_x.detach(), em.detach(), 8)[0]
res["script"] = float((o1 - o2).abs().max())
print(json.dumps(res))
""")
    for key in ("torch.float64", "torch.float32"):
        e1, e2, e3, tol = out[key]
        assert e1 <= tol and e2 <= tol and e3 <= tol, (key, out[key])
    assert out["script"] == 0.0
    assert out["gradgrad_rel"] <= 1e-12, out["gradgrad_rel"]
