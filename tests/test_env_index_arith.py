"""Host check of an arithmetic claim the neighbour-search kernel relies on
(dpmd-public_gb300/csrc/env.cu, k_nlist_env): the stencil offsets of flat
index q are formed with FP32 reciprocal multiplies, floor((q + 1/2) * fl(1/d)),
instead of integer divisions.  That is exact while q + 1/2 < 2^22, which
covers every stencil the kernel can meet (reach up to 7 cells or half cells
either way, so at most 15^3 positions); the check runs the same FP32
operations in numpy over all of them."""

import numpy as np


def test_stencil_offsets_from_fp32_reciprocals_are_exact():
    one, half = np.float32(1), np.float32(0.5)
    for hx in range(1, 8):
        for hy in range(1, 8):
            for hz in range(1, 8):
                sy, sz = 2 * hy + 1, 2 * hz + 1
                nst = (2 * hx + 1) * sy * sz
                inv_z, inv_yz = one / np.float32(sz), one / np.float32(sy * sz)
                q = np.arange(nst, dtype=np.int64)
                q0 = ((q.astype(np.float32) + half) * inv_yz).astype(np.int64)
                rq = q - q0 * sy * sz
                q1 = ((rq.astype(np.float32) + half) * inv_z).astype(np.int64)
                q2 = rq - q1 * sz
                np.testing.assert_array_equal(q0, q // (sy * sz))
                np.testing.assert_array_equal(q1, (q // sz) % sy)
                np.testing.assert_array_equal(q2, q % sz)
