"""Host side of the tensor-core embedding: the BF16 operand images the
kernels stage (rounding and the 128-byte swizzled K-major layout)."""

import importlib

import numpy as np
import torch


def _se_a(gb):
    return importlib.import_module("dpmd_public_gb300.se_a")


def test_bf16_rounding_matches_torch(gb):
    se_a = _se_a(gb)
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 4096), rng.normal(0, 1e-3, 1024),
                        [0.0, -0.0, 1.0, 3.0e38, -1e-40]]).astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(se_a._bf16_bits(x), want)


def _decode(img: bytes, nrows: int, k: int) -> np.ndarray:
    """Inverse of the swizzled image: [nrows, k] of bf16 values as float."""
    nch = (k + 63) // 64
    bits = np.frombuffer(img, np.uint16).reshape(nch, nrows, 8, 8)
    out = np.empty((nch, nrows, 8, 8), np.uint16)
    rows = np.arange(nrows)
    for p in range(8):
        out[:, :, p, :] = bits[:, rows, p ^ (rows & 7), :]
    vals = out.transpose(1, 0, 2, 3).reshape(nrows, nch * 64)
    return (vals.astype(np.uint32) << 16).view(np.float32)[:, :k]


def test_sw128_image_layout(gb):
    se_a = _se_a(gb)
    rng = np.random.default_rng(1)
    for n, k, rows in ((50, 25, 64), (100, 50, 128), (50, 100, 64), (25, 50, 64)):
        m = rng.normal(0, 1, (n, k)).astype(np.float32)
        img = se_a._sw128_image(m, rows)
        assert len(img) == ((k + 63) // 64) * rows * 128
        dec = _decode(img, rows, k)
        ref = torch.from_numpy(m).to(torch.bfloat16).float().numpy()
        assert np.array_equal(dec[:n], ref)
        assert not dec[n:].any()
    # piece p of row r sits at piece p ^ (r & 7) of that row
    m = np.zeros((8, 64), np.float32)
    m[3, 8:16] = 1.0  # row 3, piece 1
    raw = np.frombuffer(se_a._sw128_image(m, 8), np.uint16).reshape(8, 8, 8)
    assert (raw[3, 1 ^ 3] == 0x3F80).all() and raw.sum() == 8 * 0x3F80


def test_embed_tc_images_block(gb):
    se_a = _se_a(gb)
    mdl = importlib.import_module("dpmd_public_gb300.model")
    cfg = mdl.SeAConfig()
    params = mdl.init_params(cfg, 3)
    assert se_a._emb_tc_ok(cfg, params["emb"])
    img = se_a.embed_tc_images(params["emb"])
    assert img.shape == (len(params["emb"]), 51200)
    l1, l2, l3 = params["emb"][1]
    par = img[1, se_a._NET_PAR:se_a._NET_PAR + 1280].view(np.float32)
    np.testing.assert_array_equal(par[:25], np.float32(l1["w"][0]))
    np.testing.assert_array_equal(par[192:292], np.float32(l3["b"]))
    w3t = _decode(img[1, se_a._NET_B3:se_a._NET_B3 + 16384].tobytes(), 128, 50)
    np.testing.assert_array_equal(w3t[:100], torch.tensor(np.float32(l3["w"]).T).bfloat16().float())
