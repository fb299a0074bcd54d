"""The C-ABI library loads and exports every entry point include/gbdp.h
declares; host-only planning matches the reference cell geometry.  CPU only
(no compute call needs a GPU here)."""

import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gbdp.h")).read()
    return sorted(set(re.findall(r"GBDP_API\s+[\w\s\*]+?\b(gbdp_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(gb):
    lib = gb._lib.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes signature table covers exactly the header
    assert sorted(gb._lib.declared_symbols()) == names


def _declared_params():
    """name -> (return type, number of parameters) of every GBDP_API function."""
    src = open(os.path.join(ROOT, "include", "gbdp.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    out = {}
    for m in re.finditer(r"GBDP_API\s+([\w\s\*]+?)\b(gbdp_\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.S):
        ret, name, params = m.group(1).strip(), m.group(2), " ".join(m.group(3).split())
        n = 0 if params in ("", "void") else params.count(",") + 1
        out[name] = (ret, n)
    return out


def test_binding_signatures_match_the_header(gb):
    """Every ctypes signature in the binding has the header's parameter count
    and a matching return kind, so that an ABI change on one side cannot go
    unnoticed on the other."""
    sigs = gb._lib._SIGS
    decl = _declared_params()
    assert set(decl) == set(sigs)
    for name, (ret, n) in decl.items():
        restype, argtypes = sigs[name]
        assert len(argtypes) == n, (name, len(argtypes), n)
        if ret == "void":
            assert restype is None, name
        elif ret == "int":
            assert restype is ctypes.c_int, name
        elif ret == "size_t":
            assert restype is ctypes.c_size_t, name


def test_version_and_error_string(gb):
    lib = gb._lib.load()
    assert lib.gbdp_version() >= 100
    assert isinstance(lib.gbdp_last_error(), bytes)


def test_invalid_arguments_are_reported_not_raised(gb):
    lib = gb._lib.load()
    info = (ctypes.c_float * 6)(0, 1, 2, 0.1, 0.1, -1)
    rc = lib.gbdp_tabulate_fusion_se_a_f32(None, None, info, None, None, 4, 4, 0, 1, None)
    assert rc == gb._lib.GBDP_OK - 1
    assert b"last_layer_size" in lib.gbdp_last_error()
    # zero-sized work is a no-op that needs no device
    rc = lib.gbdp_tabulate_fusion_se_a_f32(None, None, info, None, None, 0, 4, 8, 1, None)
    assert rc == 0


def _plan(gb, nloc, boxes, rcut=6.0):
    L = gb._lib
    plan = L.NbrPlan()
    nf = len(nloc)
    frames = (L.NbrFrame * nf)()
    nl = np.asarray(nloc, np.int32)
    bx = np.ascontiguousarray(np.asarray(boxes, np.float64).reshape(nf, 9))
    rc = L.load().gbdp_nbr_plan_make(ctypes.byref(plan), frames, nf,
                                     nl.ctypes.data_as(ctypes.c_void_p),
                                     bx.ctypes.data_as(ctypes.c_void_p), ctypes.c_float(rcut), 0)
    return rc, plan, frames


def test_plan_geometry_and_ghost_bound(gb, oracle):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    cases = [(4, 12.42, 1), (2, 6.2, 3), (8, 24.84, 5), (16, 49.68, 9)]
    frames_in = [water.water_frame(n, L, s) for n, L, s in cases]
    rc, plan, frames = _plan(gb, [len(t) for _, t, _ in frames_in], [b for _, _, b in frames_in])
    assert rc == 0
    off = 0
    for f, (c, t, b) in enumerate(frames_in):
        fr = frames[f]
        L = b[0]
        nc = max(1, int(L / 6.0))
        assert list(fr.ncell) == [nc] * 3
        assert list(fr.ngcell) == [int(6.0 / (L / nc)) + 1] * 3
        assert fr.atom_off == off
        off += len(t)
        ec, et, em = oracle.copy_coord(c, t, b, 6.0)
        assert len(et) <= fr.ext_cap  # the reserved bound holds
    assert plan.nloc_total == off
    assert plan.ext_total == sum(frames[f].ext_cap for f in range(len(cases)))


def test_plan_rejects_bad_input(gb):
    rc, _, _ = _plan(gb, [10], np.zeros(9))
    assert rc < 0
    assert b"zero-volume" in gb._lib.load().gbdp_last_error()


def test_workspace_sizes(gb):
    L = gb._lib
    rc, plan, frames = _plan(gb, [192], np.diag([12.42] * 3))
    w32 = L.load().gbdp_env_workspace_bytes(ctypes.byref(plan), 0)
    w64 = L.load().gbdp_env_workspace_bytes(ctypes.byref(plan), 1)
    assert 0 < w32 < w64
    assert L.load().gbdp_prod_workspace_bytes(1, 192, 192, 138, 0) > 0
    assert (L.load().gbdp_prod_workspace_bytes(1, 192, 192, 138, 1)
            > L.load().gbdp_prod_workspace_bytes(1, 192, 192, 138, 0))


def test_fitting_tc_argument_errors(gb):
    """The tensor-core fitting's argument checks run before any device work:
    a row block that is not 128-aligned, missing column scales, a non-positive
    activation scale and a null D row-scale array are reported, not raised."""
    L = gb._lib
    lib = L.load()
    nets = (L.FitTcNet * 1)()
    fake = ctypes.c_void_p(256)  # never dereferenced: the checks fail first
    for l in range(3):
        nets[0].w_hi[l] = nets[0].w_lo[l] = nets[0].wt_hi[l] = nets[0].wt_lo[l] = fake
        nets[0].b[l] = fake
        nets[0].cs_fwd[l] = nets[0].cs_bwd[l] = fake
    nets[0].idt[1] = nets[0].idt[2] = nets[0].w_out = fake
    for a in range(5):
        nets[0].act_scale[a] = 1.0
    nrows = (ctypes.c_int * 1)(100)
    ws = ctypes.c_void_p(512)

    def call(row_off, rscale=fake):
        ro = (ctypes.c_int * 2)(*row_off)
        return lib.gbdp_fitting_tc_f32(fake, fake, fake, fake, rscale, 1, nrows, ro, nets, ws,
                                       ctypes.c_size_t(1 << 30), None)

    assert call([0, 100]) != 0 and b"multiple of 128" in lib.gbdp_last_error()
    assert call([0, 128], rscale=None) != 0 and b"null argument" in lib.gbdp_last_error()
    nets[0].act_scale[2] = 0.0
    assert call([0, 128]) != 0 and b"act_scale" in lib.gbdp_last_error()
    nets[0].act_scale[2] = 1.0
    nets[0].cs_bwd[1] = None
    assert call([0, 128]) != 0 and b"column scales" in lib.gbdp_last_error()


def test_descriptor_split_needs_row_scales(gb):
    lib = gb._lib.load()
    fake = ctypes.c_void_p(256)
    sel = (ctypes.c_int * 2)(46, 92)
    info = (ctypes.c_float * 12)(*([0, 1, 2, 0.1, 0.1, -1] * 2))
    tabs = (ctypes.c_void_p * 2)(fake, fake)
    rc = lib.gbdp_se_a_descriptor_fwd_split_f32(fake, fake, fake, None, fake, fake, None, tabs,
                                               info, 2, sel, 1, 8, 100, 16, None)
    assert rc != 0 and b"D_rscale" in lib.gbdp_last_error()
