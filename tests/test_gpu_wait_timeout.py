"""A bounded device wait that runs out: the self-test kernel of the C ABI
(gbdp_selftest_wait_timeout) completes one mbarrier phase with a bulk copy,
then waits on a phase that nothing completes with a small poll limit.  The
wait gives up, the status word reads GBDP_STATUS_TIMEOUT, the kernel
returns, and the context keeps working (a library kernel runs afterwards and
gives its usual result)."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.mark.parametrize("limit", [1, 1000])
def test_wait_gives_up_and_reports_timeout(gb, limit):
    gb.load_library()
    L = gb._lib.load()
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    result = torch.tensor([41, 7, 0, 0], dtype=torch.int32, device=DEV)
    assert result.data_ptr() % 16 == 0
    rc = L.gbdp_selftest_wait_timeout(ctypes.c_void_p(status.data_ptr()),
                                      ctypes.c_void_p(result.data_ptr()), limit,
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, L.gbdp_last_error()
    torch.cuda.synchronize()
    assert int(status[0]) == 3  # GBDP_STATUS_TIMEOUT
    assert result[0].item() == 42 and result[1].item() == 0
    # the context is healthy: a library kernel runs and is right
    water = __import__("dpmd_public_gb300.water", fromlist=["x"])
    c, t, b = water.water_frame(2, 6.2, 7)
    plan = gb.NeighborPlan([len(t)], b[None], 6.0, DEV, torch.float64)
    avg = torch.zeros((2, 552), dtype=torch.float64, device=DEV)
    std = torch.ones((2, 552), dtype=torch.float64, device=DEV)
    r = gb.env_mat_packed(plan, torch.tensor(c, device=DEV), torch.tensor(t, device=DEV), avg, std,
                          0.5, [46, 92])
    import oracle as O

    em, emd, rij, nl = O.prod_env_mat_a_pbc(c, t, b, avg.cpu().numpy(), std.cpu().numpy(), 6.0,
                                            0.5, [46, 92])
    assert np.array_equal(r.nlist.cpu().numpy().reshape(-1), nl)


def test_selftest_rejects_bad_arguments(gb):
    gb.load_library()
    L = gb._lib.load()
    buf = torch.zeros(8, dtype=torch.int32, device=DEV)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.gbdp_selftest_wait_timeout(ctypes.c_void_p(buf.data_ptr()),
                                        ctypes.c_void_p(buf.data_ptr() + 16), 0, st) < 0
    assert b"limit" in L.gbdp_last_error()
    assert L.gbdp_selftest_wait_timeout(ctypes.c_void_p(buf.data_ptr()),
                                        ctypes.c_void_p(buf.data_ptr() + 4), 5, st) < 0
    assert b"aligned" in L.gbdp_last_error()
