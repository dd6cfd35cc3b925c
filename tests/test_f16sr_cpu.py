"""Stochastic rounding of the FP16 offset storage (NGB_STORE_F16SR) in the
oracle: bit for bit against the GPU's cvt.rs.f16x2.f32 (committed golden
vectors, tests/golden/make_f16_rs_golden.cu), the round-toward-zero
conversion against an exact numpy model, the unbiasedness of the dithered
store, and the spread of the dither bits."""
import ctypes
import os

import numpy as np

from helpers import P


def _rz_model(x):
    """float32 -> float16 rounded toward zero, from numpy's nearest rounding."""
    h = x.astype(np.float16)
    hb = h.view(np.uint16).copy()
    over = np.abs(h.astype(np.float32)) > np.abs(x)  # nearest rounded away from zero: step back one ulp
    hb[over] -= 1
    return hb


def test_zero_random_bits_round_toward_zero(orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.standard_normal(200000).astype(np.float32) * s
                        for s in (1e-7, 1e-5, 1e-3, 1.0, 300.0, 6e4)] + [np.float32([0.0, -0.0, 65504.0, -65519.0])])
    x = x[np.abs(x) < 65536.0]  # from 2^16 on the conversion overflows to infinity (golden test below)
    r = np.zeros(x.size, np.uint32)
    out = np.zeros(x.size, np.uint16)
    orc.orc_f32_to_f16_sr(P(x), P(r), P(out), x.size)
    assert np.array_equal(out, _rz_model(x))


def test_dithered_store_is_unbiased(orc):
    """A value between two FP16 numbers rounds up with probability equal to
    its remainder: the mean of many dithered stores is the value itself."""
    rng = np.random.default_rng(2)
    for v in (0.1234567, -3.3333333e-3, 17.77777, 1.0e-4 + 3e-9, 3.3e-6, -4.1e-7):
        x = np.full(1 << 16, v, np.float32)
        r = rng.integers(0, 1 << 13, x.size, dtype=np.uint32)
        out = np.zeros(x.size, np.uint16)
        orc.orc_f32_to_f16_sr(P(x), P(r), P(out), x.size)
        got = out.view(np.float16).astype(np.float64).mean()
        ulp = abs(float(np.spacing(np.float16(v))))
        assert abs(got - float(np.float32(v))) < 0.02 * ulp, (v, got)


def test_dither_bits_are_spread(orc):
    n = 1 << 16
    cell = np.arange(n, dtype=np.uint64) * np.uint64(37) + np.uint64(1 << 33)
    q = (np.arange(n) % 19).astype(np.int32)
    out = np.zeros(n, np.uint32)
    orc.orc_dither_bits(cell.ctypes.data_as(ctypes.c_void_p), q.ctypes.data_as(ctypes.c_void_p), 5, P(out), n)
    assert out.max() < (1 << 13)
    hist = np.bincount(out >> 9, minlength=16)  # 16 bins of the 13-bit range
    assert hist.min() > 0.8 * n / 16 and hist.max() < 1.2 * n / 16


def test_matches_gpu_stochastic_rounding_golden(orc):
    """The oracle's conversion equals the hardware's on every committed case:
    the one-bit scan (bits 0-12 of the random word feed the low result, 16-28
    the high one, each at weight 2^-13 ulp) and seeded random values of both
    signs, a quarter of them in the FP16 subnormal range."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "f16_rs_golden.bin")
    raw = np.fromfile(path, np.uint8)
    n = int(raw[:4].view(np.int32)[0])
    body = raw[4:].view(np.uint32).reshape(4, n)
    a, b, r, out = body[0].view(np.float32).copy(), body[1].view(np.float32).copy(), body[2], body[3]
    assert n >= 16384 and ((np.abs(a) < 2.0 ** -14) & (a != 0)).sum() > 3000
    rh = ((r >> 16) & 0x1FFF).astype(np.uint32)
    rl = (r & 0x1FFF).astype(np.uint32)
    oh = np.zeros(n, np.uint16)
    ol = np.zeros(n, np.uint16)
    orc.orc_f32_to_f16_sr(P(a), P(rh), P(oh), n)
    orc.orc_f32_to_f16_sr(P(b), P(rl), P(ol), n)
    assert np.array_equal(oh, (out >> 16).astype(np.uint16)), int((oh != (out >> 16)).sum())
    assert np.array_equal(ol, (out & 0xFFFF).astype(np.uint16)), int((ol != (out & 0xFFFF)).sum())
