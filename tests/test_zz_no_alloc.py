"""The allocation-free environment-matrix entry point.

Some callers cannot allocate device memory when they call us: an MD engine
that owns all device memory through its own pool and forbids allocations in
its force callback, or code running while a stream is being captured.
gbdp_prod_env_mat_a_noalloc_f32 serves them from a built-in device scratch
array.  This file is collected last on purpose: if it fails, a run that stops
at the first failure has already run every other test.

Checks, through the C ABI: two calls in a row (different frames, so the
second call must not see the first call's state) match the workspace-based
entry point exactly for the integer outputs and within the fp32 env
tolerance of tests/test_gpu_env.py for the rest; an oversize batch is
rejected with a message before any device work."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
SEL = [46, 92]
NNEI = sum(SEL)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stats():
    rng = np.random.default_rng(4)
    avg = np.zeros((2, NNEI * 4), np.float32)
    avg[:, 0::4] = rng.uniform(0.05, 0.15, (2, NNEI))
    std = np.ones((2, NNEI * 4), np.float32)
    std[:, 0::4] = rng.uniform(0.1, 0.2, (2, NNEI))
    std[:, 1::4] = std[:, 2::4] = std[:, 3::4] = rng.uniform(0.05, 0.1, (2, NNEI))
    return avg, std


def _noalloc_call(gb, plan, coord, atype, avg, std):
    L = gb._lib
    n, ext = plan.nloc_total, plan.ext_total
    out = {
        "em": torch.empty((n, NNEI, 4), dtype=torch.float32, device=DEV),
        "em_deriv": torch.empty((n, NNEI, 4, 3), dtype=torch.float32, device=DEV),
        "rij": torch.empty((n, NNEI, 3), dtype=torch.float32, device=DEV),
        "nlist": torch.empty((n, NNEI), dtype=torch.int32, device=DEV),
        "nlist_ext": torch.empty((n, NNEI), dtype=torch.int32, device=DEV),
        "ext_coord": torch.empty((ext, 3), dtype=torch.float32, device=DEV),
        "ext_type": torch.empty((ext,), dtype=torch.int32, device=DEV),
        "ext_map": torch.empty((ext,), dtype=torch.int32, device=DEV),
        "ext_nall": torch.empty((plan.nframes,), dtype=torch.int32, device=DEV),
        "status": torch.full((1,), -7, dtype=torch.int32, device=DEV),
    }
    sel = (ctypes.c_int * 2)(*SEL)
    rc = L.load().gbdp_prod_env_mat_a_noalloc_f32(
        _ptr(out["em"]), _ptr(out["em_deriv"]), _ptr(out["rij"]), _ptr(out["nlist"]),
        _ptr(out["nlist_ext"]), _ptr(out["ext_coord"]), _ptr(out["ext_type"]), _ptr(out["ext_map"]),
        _ptr(out["ext_nall"]), _ptr(out["status"]), _ptr(coord), _ptr(atype), _ptr(avg), _ptr(std),
        ctypes.byref(plan.plan), plan.frames_host, ctypes.c_float(0.5), sel, 2,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, out


def test_noalloc_matches_workspace_entry_twice(gb):
    gb.load_library()
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    avg_n, std_n = _stats()
    avg = torch.tensor(avg_n, device=DEV)
    std = torch.tensor(std_n, device=DEV)
    for frames in ([water.water_frame(4, 12.42, 61)],
                   water.ragged_frames(3, seed=62, lo=20, hi=150)):
        coord = torch.tensor(np.concatenate([f[0] for f in frames]), dtype=torch.float32, device=DEV)
        atype = torch.tensor(np.concatenate([f[1] for f in frames]), dtype=torch.int32, device=DEV)
        plan = gb.NeighborPlan([len(f[1]) for f in frames], np.stack([f[2] for f in frames]), 6.0, DEV,
                               torch.float32)
        rc, out = _noalloc_call(gb, plan, coord, atype, avg, std)
        assert rc == 0, gb._lib.load().gbdp_last_error()
        ref = gb.env_mat_packed(plan, coord, atype, avg, std, 0.5, SEL, need_nlist_ext=True)
        torch.cuda.synchronize()
        assert int(out["status"][0]) == 0
        assert torch.equal(out["nlist"], ref.nlist)
        assert torch.equal(out["nlist_ext"], ref.nlist_ext)
        assert torch.equal(out["ext_nall"], ref.ext_nall)
        for f in range(plan.nframes):
            eo, n = int(plan.ext_off[f]), int(ref.ext_nall[f])
            assert torch.equal(out["ext_coord"][eo:eo + n], ref.ext_coord[eo:eo + n])
            assert torch.equal(out["ext_map"][eo:eo + n], ref.ext_map[eo:eo + n])
        torch.testing.assert_close(out["em"], ref.em, atol=5e-6, rtol=5e-6)
        torch.testing.assert_close(out["em_deriv"], ref.em_deriv, atol=2e-5, rtol=2e-5)
        torch.testing.assert_close(out["rij"], ref.rij, atol=5e-6, rtol=5e-6)


def test_noalloc_rejects_batches_beyond_the_scratch(gb):
    gb.load_library()
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    c, t, b = water.water_frame(48, 149.04, 63)  # 331,776 atoms: workspace > 16 MiB
    plan = gb.NeighborPlan([len(t)], b[None], 6.0, DEV, torch.float32)
    coord = torch.zeros((1, 3), dtype=torch.float32, device=DEV)
    atype = torch.zeros((1,), dtype=torch.int32, device=DEV)
    avg = torch.zeros((2, NNEI * 4), dtype=torch.float32, device=DEV)
    rc, out = _noalloc_call(gb, plan, coord, atype, avg, avg)
    assert rc < 0
    assert b"scratch" in gb._lib.load().gbdp_last_error()


def _small_frames(n, seed):
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    return [water.water_frame(2, 6.2, seed + k) for k in range(n)]


def _inputs(gb, frames, pinned_frames=False):
    coord = torch.tensor(np.concatenate([f[0] for f in frames]), dtype=torch.float32, device=DEV)
    atype = torch.tensor(np.concatenate([f[1] for f in frames]), dtype=torch.int32, device=DEV)
    plan = gb.NeighborPlan([len(f[1]) for f in frames], np.stack([f[2] for f in frames]), 6.0, DEV,
                           torch.float32)
    return coord, atype, plan


def test_noalloc_frame_table_limit_is_234_frames(gb):
    """The built-in frame table holds 234 frame records (64 KiB / 280 B): a
    234-frame batch runs and matches the workspace entry point, a 235-frame
    batch is rejected with a message before any device work."""
    gb.load_library()
    avg_n, std_n = _stats()
    avg = torch.tensor(avg_n, device=DEV)
    std = torch.tensor(std_n, device=DEV)
    assert ctypes.sizeof(gb._lib.NbrFrame) == 280
    frames = _small_frames(235, 700)
    coord, atype, plan = _inputs(gb, frames)
    rc, out = _noalloc_call(gb, plan, coord, atype, avg, std)
    assert rc < 0
    assert b"frame table" in gb._lib.load().gbdp_last_error()
    assert int(out["status"][0]) == -7  # nothing ran: the status word is untouched
    coord, atype, plan = _inputs(gb, frames[:234])
    rc, out = _noalloc_call(gb, plan, coord, atype, avg, std)
    assert rc == 0, gb._lib.load().gbdp_last_error()
    ref = gb.env_mat_packed(plan, coord, atype, avg, std, 0.5, SEL, need_nlist_ext=True)
    torch.cuda.synchronize()
    assert int(out["status"][0]) == 0
    assert torch.equal(out["nlist"], ref.nlist)
    torch.testing.assert_close(out["em"], ref.em, atol=5e-6, rtol=5e-6)


def test_noalloc_rejected_call_leaves_the_scratch_alone(gb):
    """A call that an argument check rejects (ntypes out of range) returns
    an error and enqueues nothing, so an earlier call's frame table and
    results stay intact."""
    gb.load_library()
    avg_n, std_n = _stats()
    avg = torch.tensor(avg_n, device=DEV)
    std = torch.tensor(std_n, device=DEV)
    coord, atype, plan = _inputs(gb, _small_frames(3, 710))
    rc, out = _noalloc_call(gb, plan, coord, atype, avg, std)
    assert rc == 0
    torch.cuda.synchronize()
    L = gb._lib.load()
    bad = dict(out)
    bad["status"] = torch.full((1,), -7, dtype=torch.int32, device=DEV)
    sel = (ctypes.c_int * 2)(*SEL)
    rc = L.gbdp_prod_env_mat_a_noalloc_f32(
        *[_ptr(bad[k]) for k in ("em", "em_deriv", "rij", "nlist", "nlist_ext", "ext_coord",
                                 "ext_type", "ext_map", "ext_nall", "status")],
        _ptr(coord), _ptr(atype), _ptr(avg), _ptr(std), ctypes.byref(plan.plan), plan.frames_host,
        ctypes.c_float(0.5), sel, 0, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc < 0 and b"ntypes" in L.gbdp_last_error()
    torch.cuda.synchronize()
    assert int(bad["status"][0]) == -7


def test_noalloc_call_captured_in_a_cuda_graph(gb):
    """One uncaptured call, then the same call captured in a CUDA graph with
    the frame table in pinned host memory: every replay reproduces the
    uncaptured outputs."""
    gb.load_library()
    avg_n, std_n = _stats()
    avg = torch.tensor(avg_n, device=DEV)
    std = torch.tensor(std_n, device=DEV)
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    frames = water.ragged_frames(4, seed=720, lo=20, hi=120)
    coord, atype, plan = _inputs(gb, frames)
    rc, first = _noalloc_call(gb, plan, coord, atype, avg, std)
    assert rc == 0
    torch.cuda.synchronize()
    raw = bytes(plan.frames_host)
    pinned = torch.frombuffer(bytearray(raw), dtype=torch.uint8).pin_memory()
    L = gb._lib.load()
    n, ext = plan.nloc_total, plan.ext_total
    out = {k: torch.empty_like(v) for k, v in first.items()}
    sel = (ctypes.c_int * 2)(*SEL)
    keys = ("em", "em_deriv", "rij", "nlist", "nlist_ext", "ext_coord", "ext_type", "ext_map",
            "ext_nall", "status")
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            rc = L.gbdp_prod_env_mat_a_noalloc_f32(
                *[_ptr(out[k]) for k in keys], _ptr(coord), _ptr(atype), _ptr(avg), _ptr(std),
                ctypes.byref(plan.plan), ctypes.c_void_p(pinned.data_ptr()), ctypes.c_float(0.5),
                sel, 2, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.current_stream().wait_stream(side)
    assert rc == 0, L.gbdp_last_error()
    for _ in range(2):
        for v in out.values():
            v.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert int(out["status"][0]) == 0
        for k in ("nlist", "nlist_ext", "ext_nall"):
            assert torch.equal(out[k], first[k]), k
        for k in ("em", "em_deriv", "rij"):
            assert torch.equal(out[k], first[k]), k
