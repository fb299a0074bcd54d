"""The reference's own PyTorch descriptor, replayed through this library.

tests/golden/ref_descriptor_pt.npz holds what the reference's DescrptSeA
(deepmd/pt/model/descriptor/se_a.py:316-380, compressed, FP64, its own
tabulate_fusion_se_a compiled from source/op/pt/tabulate_multi_device.cc)
computed on CPU for a seeded 192-atom water frame that its own
extend_input_and_build_neighbor_list (deepmd/pt/utils/nlist.py:14-46)
extended and listed, with seeded weights and statistics (made by
tests/golden/make_golden.py).  On the GPU:

* the tables this library builds for those weights have the reference's
  range and row count, and its coefficient magnitude to 1e-6;
* every tabulate_fusion_se_a call the reference module made, replayed
  through torch.ops.deepmd.tabulate_fusion_se_a on CUDA: outputs and the
  input gradients for the recorded output gradient within 1e-10;
* the whole descriptor from the reference's extended coordinates and
  neighbour list (prod_env_mat_a_nlist, the tabulated embedding and G^T R
  of the operator form): within 1e-10 of the reference's, and the gradient
  of the same seeded linear function of it wrt the extended coordinates
  (autograd to the env matrix, then prod_force_se_a) within 1e-9.
"""

import importlib
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ref(gb):
    gb.load_library()
    g = dict(np.load(os.path.join(HERE, "golden", "ref_descriptor_pt.npz")))
    mdl = importlib.import_module("dpmd_public_gb300.model")
    cfg = mdl.SeAConfig()
    params = mdl.init_params(cfg, int(g["seed"]))
    tabs, infos = mdl.build_tables(params, g["davg"], g["dstd"], float(g["rmin"]), cfg)
    return g, cfg, params, tabs, infos


def test_tables_match_the_reference_modules(ref):
    g, cfg, params, tabs, infos = ref
    for q in range(int(g["ncalls"])):
        np.testing.assert_array_equal(infos[q], g[f"call{q}_info"])
        assert tabs[q].shape[0] == int(g[f"call{q}_table_rows"])
        # the sum is dominated by the a3..a5 columns, which carry the nodes'
        # rounding amplified by 1 / stride^n in any evaluation order (the
        # interpolants themselves agree to 1e-13: test_host_model.py)
        np.testing.assert_allclose(np.abs(tabs[q]).sum(), float(g[f"call{q}_table_abs_sum"]),
                                   rtol=1e-6)


def test_replayed_tabulate_calls(ref):
    g, cfg, params, tabs, infos = ref
    for q in range(int(g["ncalls"])):
        table = torch.tensor(tabs[q], device=DEV)
        info = torch.tensor(g[f"call{q}_info"])  # on the host, as the module passes it
        ex = torch.tensor(g[f"call{q}_em_x"], device=DEV).requires_grad_(True)
        em = torch.tensor(g[f"call{q}_em"], device=DEV).requires_grad_(True)
        out = torch.ops.deepmd.tabulate_fusion_se_a(table, info, ex, em, int(g[f"call{q}_last"]))[0]
        ref_out = g[f"call{q}_out"]
        scale = np.abs(ref_out).max()
        assert np.abs(out.detach().cpu().numpy() - ref_out).max() <= 1e-10 * scale
        gx, gm = torch.autograd.grad(out, (ex, em), torch.tensor(g[f"call{q}_dy"], device=DEV))
        for a, b in ((gx, g[f"call{q}_gx"]), (gm, g[f"call{q}_gm"])):
            assert np.abs(a.cpu().numpy() - b).max() <= 1e-10 * max(np.abs(b).max(), 1.0)


def test_descriptor_and_coordinate_gradient(gb, ref):
    g, cfg, params, tabs, infos = ref
    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    ops = importlib.import_module("dpmd_public_gb300.ops")
    m = se_a.SeAModel(cfg, params, g["davg"], g["dstd"], DEV, torch.float64, tabs, infos)
    ext = torch.tensor(g["ext_coord"], device=DEV)
    et = torch.tensor(g["ext_atype"], device=DEV)
    nloc = len(g["atype"])
    nall = ext.shape[0]
    em, emd, rij, nl = torch.ops.deepmd.prod_env_mat_a_nlist(
        ext.reshape(1, -1), et.reshape(1, -1), torch.tensor(g["nlist"], device=DEV)[None],
        m.davg, m.dstd, cfg.rcut, cfg.rcut_smth, list(cfg.sel))
    em = em.reshape(nloc, cfg.nnei, 4).detach().requires_grad_(True)
    D = m._descriptor_from_em(em, et[:nloc].to(torch.int32), compressed=True)
    Dn = D.detach().cpu().numpy()
    head = g["desc_head"]
    assert np.abs(Dn[: len(head)] - head).max() <= 1e-10 * np.abs(head).max()
    np.testing.assert_allclose(np.linalg.norm(Dn, axis=1), g["desc_norm"], rtol=1e-10)
    wts = np.random.default_rng(int(g["seed"]) + 2).normal(0, 1, (1, nloc, D.shape[1]))[0]
    (net,) = torch.autograd.grad((D * torch.tensor(wts, device=DEV)).sum(), em)
    natoms = torch.tensor([nloc, nall, 0, 0], dtype=torch.int32)
    force = ops.prod_force_se_a_impl(net.reshape(1, -1), emd, nl, natoms, cfg.nnei, 0)
    grad = -force.reshape(nall, 3).cpu().numpy()
    assert np.abs(grad - g["grad_ext"]).max() <= 1e-9
