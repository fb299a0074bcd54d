"""Pin the CPU oracle (oracle/oracle.cc) to the reference's own known-answer
vectors (source/lib/tests/*.cc, source/tests/pt/test_tabulate_fusion_se_a.py)
and to fixtures produced by the reference's CPU library (ref_water.npz).
CPU only."""

import numpy as np
import pytest


def _sec_sel(sec):
    return [sec[i + 1] - sec[i] for i in range(len(sec) - 1)]


def _fixture_env(O, fx, dtype=np.float64):
    """copy_coord + format + env mat of the reference's 6-atom fixture
    (13 A box), as test_env_mat_a.cc / test_prod_force_a.cc SetUp do."""
    posi = np.array(fx["posi"], dtype)
    atype = np.array(fx["atype"], np.int32)
    box = np.array(fx["box"], dtype)
    sel = _sec_sel(fx["sec_a"])
    ec, et, emap = O.copy_coord(posi, atype, box, fx["rc"])
    nloc = len(atype)
    nnei = sum(sel)
    avg = np.zeros((2, nnei * 4), dtype)
    std = np.ones((2, nnei * 4), dtype)
    em, emd, rij, nl = O.prod_env_mat_a_ext(ec, et, nloc, avg, std, fx["rc"], fx["rc_smth"], sel)
    return dict(nloc=nloc, nall=len(et), nnei=nnei, em=em, emd=emd, rij=rij, nl=nl,
                ec=ec, et=et, emap=emap, sel=sel)


@pytest.mark.parametrize("name", ["TestEnvMatA", "TestEnvMatAShortSel"])
def test_env_mat_golden(oracle, golden_lib, name):
    fx = golden_lib[name]
    r = _fixture_env(oracle, fx)
    np.testing.assert_allclose(r["em"], np.array(fx["expected_env"]), atol=1e-5)


@pytest.mark.parametrize("name", ["TestFormatNlist", "TestFormatNlistShortSel"])
def test_format_nlist_golden(oracle, golden_lib, name):
    fx = golden_lib[name]
    posi = np.array(fx["posi"])
    atype = np.array(fx["atype"], np.int32)
    ec, et, emap = oracle.copy_coord(posi, atype, np.array(fx["box"]), fx["rc"])
    nl = oracle.format_nlist(ec, et, len(atype), fx["rc"], _sec_sel(fx["sec_a"]))
    np.testing.assert_array_equal(nl.reshape(-1), np.array(fx["expect_nlist_cpy"]))


def test_prod_force_golden(oracle, golden_lib):
    fx = golden_lib["TestProdForceA"]
    r = _fixture_env(oracle, fx)
    nd = r["nloc"] * r["nnei"] * 4
    net = 10 - np.arange(nd) * 0.01
    nf = fx["nframes"]
    f = oracle.prod_force_a(np.tile(net, nf), np.tile(r["emd"], nf), np.tile(r["nl"], nf),
                            r["nloc"], r["nall"], r["nnei"], nf)
    exp = np.tile(np.array(fx["expected_force"]), nf)
    np.testing.assert_allclose(f.reshape(-1), exp, atol=1e-5)


def test_prod_virial_golden(oracle, golden_lib):
    fx = golden_lib["TestProdVirialA"]
    r = _fixture_env(oracle, fx)
    nd = r["nloc"] * r["nnei"] * 4
    net = 10 - np.arange(nd) * 0.01
    v, av = oracle.prod_virial_a(net, r["emd"], r["rij"], r["nl"], r["nloc"], r["nall"], r["nnei"])
    np.testing.assert_allclose(v, np.array(fx["expected_virial"]), atol=1e-5)
    np.testing.assert_allclose(av, np.array(fx["expected_atom_virial"]), atol=1e-5)


def test_prod_force_grad_golden(oracle, golden_lib):
    fx = golden_lib["TestProdForceGradA"]
    r = _fixture_env(oracle, fx)
    nf = fx["nframes"]
    grad = 10 - np.arange(r["nloc"] * 3) * 0.1
    g = oracle.prod_force_grad_a(np.tile(grad, nf), np.tile(r["emd"], nf), np.tile(r["nl"], nf),
                                 r["nloc"], r["nnei"], nf)
    np.testing.assert_allclose(g, np.tile(np.array(fx["expected_grad_net"]), nf), atol=1e-5)


def test_prod_virial_grad_golden(oracle, golden_lib):
    fx = golden_lib["TestProdVirialGradA"]
    r = _fixture_env(oracle, fx)
    grad = 10 - np.arange(9) * 1.0
    g = oracle.prod_virial_grad_a(grad, r["emd"], r["rij"], r["nl"], r["nloc"], r["nnei"])
    np.testing.assert_allclose(g, np.array(fx["expected_grad_net"]), atol=1e-5)


def test_tabulate_lib_golden(oracle, golden_lib):
    fx = golden_lib["TestTabulateSeA"]
    nloc, nnei, M = fx["nloc"], fx["nnei"], fx["last_layer_size"]
    table = np.array(fx["table"]).reshape(-1, 6 * M)
    info = np.array(fx["info"])
    em_x = np.array(fx["em_x"]).reshape(nloc * nnei, 1)
    em = np.array(fx["em"]).reshape(nloc, nnei, 4)
    out = oracle.tabulate_fusion_se_a(table, info, em_x, em, M)
    np.testing.assert_allclose(out.reshape(-1), fx["expected_xyz_scatter"], atol=1e-5)
    gx, gm = oracle.tabulate_fusion_se_a_grad(table, info, em_x, em, np.ones((nloc, 4, M)))
    np.testing.assert_allclose(gx.reshape(-1), fx["expected_dy_dem_x"], atol=1e-5)
    np.testing.assert_allclose(gm.reshape(-1), fx["expected_dy_dem"], atol=1e-5)


@pytest.mark.parametrize("dtype,prec", [(np.float64, 1e-10), (np.float32, 1e-5)])
def test_tabulate_pt_golden(oracle, golden_pt, dtype, prec):
    g = golden_pt
    M = 8
    table = np.array(g["table_tensor"]["values"], dtype).reshape(-1, 6 * M)
    info = np.array(g["table_info_tensor"]["values"], dtype)
    em_x = np.array(g["em_x_tensor"]["values"], dtype).reshape(-1, 1)
    em = np.array(g["em_tensor"]["values"], dtype).reshape(4, 4, 4)
    out = oracle.tabulate_fusion_se_a(table, info, em_x, em, M)
    exp = np.array(g["expected_descriptor_tensor"]["values"], dtype).reshape(4, 4, M)
    np.testing.assert_allclose(out, exp, atol=prec, rtol=prec)
    gx, gm = oracle.tabulate_fusion_se_a_grad(table, info, em_x, em, np.ones((4, 4, M), dtype))
    np.testing.assert_allclose(gx.reshape(-1), np.array(g["expected_dy_dem_x"]["values"], dtype),
                               atol=prec, rtol=prec)
    np.testing.assert_allclose(gm.reshape(-1), np.array(g["expected_dy_dem"]["values"], dtype),
                               atol=prec, rtol=prec)


@pytest.mark.parametrize("tag", ["w192", "w24", "w1536"])
@pytest.mark.parametrize("sfx,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_env_mat_vs_reference_run(oracle, golden_water, tag, sfx, dtype):
    """Bit-exact against the reference library's own output on seeded water."""
    g = golden_water
    sel = list(g["sel"])
    nnei = sum(sel)
    em, emd, rij, nl, ec, et, emap = oracle.prod_env_mat_a_pbc(
        g[f"{tag}_coord"].astype(dtype), g[f"{tag}_atype"], g[f"{tag}_box"].astype(dtype),
        g["avg"].astype(dtype), g["std"].astype(dtype), float(g["rcut"]), float(g["rcut_smth"]),
        sel, return_ext=True)
    np.testing.assert_array_equal(nl, g[f"{tag}_{sfx}_nlist"].astype(np.int32))
    np.testing.assert_array_equal(emap, g[f"{tag}_{sfx}_mapping"].astype(np.int32))
    assert len(et) == int(g[f"{tag}_{sfx}_nall"])
    keep = 24 * nnei
    np.testing.assert_array_equal(em[: keep * 4], g[f"{tag}_{sfx}_em"])
    np.testing.assert_array_equal(emd[: keep * 12], g[f"{tag}_{sfx}_em_deriv"])
    np.testing.assert_array_equal(rij[: keep * 3], g[f"{tag}_{sfx}_rij"])


@pytest.mark.parametrize("sfx,dt", [("f64", np.float64), ("f32", np.float32)])
def test_oracle_format_nlist_pt_matches_reference(oracle, sfx, dt):
    """The forward_lower neighbour formatting restated in the oracle equals the
    reference's own PyTorch functions (_format_nlist with the forced sort,
    nlist_distinguish_types) run on an unsorted rcut + skin candidate list."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "pt_format_nlist.npz"))
    nloc = int(g["nloc"])
    out = oracle.format_nlist_pt(g["ext_coord"].astype(dt), g["ext_type"], g["nlist_in"], nloc,
                                 float(g["rcut"]), list(g["sel"]))
    np.testing.assert_array_equal(out, g[f"{sfx}_nlist"])


def _ref_model_cases():
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_deeppot_sea.npz"))
    cases = []
    for n in range(int(g["ncases"])):
        c = g[f"case{n}_coord"].reshape(-1, 3)
        t = g[f"case{n}_atype"].astype(np.int32)
        # the non-periodic case: a box far wider than rcut has no image in range
        b = g[f"case{n}_box"] if f"case{n}_box" in g.files else np.diag([100.0] * 3).reshape(-1)
        cases.append((c, t, b, g[f"case{n}_atomic_energy"], g[f"case{n}_force"].reshape(-1, 3),
                      g[f"case{n}_atomic_virial"].reshape(-1, 9).sum(0)))
    return g, cases


def test_composite_reproduces_reference_model_testcase(gb, oracle):
    """The FP64 CPU composite with the reference's se_e2_a test model
    (deeppot_sea.yaml, loaded through the package's serialized-model reader)
    gives the atomic energies, forces and virial its own inference test
    expects (deeppot-testcase.yaml: periodic, non-periodic and elongated-box
    cases) to 1e-12."""
    import composite
    import importlib

    S = importlib.import_module("dpmd_public_gb300.serial")
    g, cases = _ref_model_cases()
    cfg, params, davg, dstd, tm = S.unflatten(dict(g))
    assert tm == ["O", "H"]
    for c, t, b, ae_ref, f_ref, v_ref in cases:
        E, F, V, ae = composite.energy_force_virial(cfg, params, davg, dstd, c, t, b)
        np.testing.assert_allclose(ae, ae_ref, rtol=0, atol=1e-12)
        np.testing.assert_allclose(F, f_ref, rtol=0, atol=1e-12)
        np.testing.assert_allclose(V.reshape(-1), v_ref, rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", ["w24", "w192", "w1536"])
@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_cell_list_build_matches_the_reference_nlist(oracle, golden_water, name, dt):
    """The O(N) cell-list candidate build (the reference's build_nlist) gives
    the neighbour list the reference library produced with its brute-force
    build_nlist_cpu, element by element, and the same env matrix."""
    g = golden_water
    dtype = np.float64 if dt == "f64" else np.float32
    sel = [int(s) for s in g["sel"]]
    c = g[f"{name}_coord"].astype(dtype)
    em, emd, rij, nl = oracle.prod_env_mat_a_pbc(
        c, g[f"{name}_atype"], g[f"{name}_box"].astype(dtype), g["avg"].astype(dtype),
        g["std"].astype(dtype), float(g["rcut"]), float(g["rcut_smth"]), sel, cell_list=True)
    np.testing.assert_array_equal(nl, g[f"{name}_{dt}_nlist"].astype(np.int32))
    n = g[f"{name}_{dt}_em"].size
    np.testing.assert_array_equal(em[:n], g[f"{name}_{dt}_em"])


def test_cell_list_build_matches_brute_force_on_ragged_frames(oracle, gb):
    """Frames of 8..512 molecules at 1 g/cm3 (boxes from 6 to 25 A, so one to
    four cells per edge): both candidate builds give the same list."""
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    sel = [46, 92]
    avg = np.zeros((2, 552))
    std = np.ones((2, 552))
    for c, t, b in water.ragged_frames(6, seed=91, lo=8, hi=512):
        for dtype in (np.float64, np.float32):
            a = oracle.prod_env_mat_a_pbc(c.astype(dtype), t, b.astype(dtype), avg.astype(dtype),
                                          std.astype(dtype), 6.0, 0.5, sel, map_to_local=False)
            b2 = oracle.prod_env_mat_a_pbc(c.astype(dtype), t, b.astype(dtype), avg.astype(dtype),
                                           std.astype(dtype), 6.0, 0.5, sel, map_to_local=False,
                                           cell_list=True)
            np.testing.assert_array_equal(a[3], b2[3])
            np.testing.assert_array_equal(a[0], b2[0])
