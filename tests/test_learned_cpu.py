"""Host side of the learned-preconditioner solver's C ABI: the weight file
(NGBUNET1, BF16 values) round trip and the argument checks of
ngb_learned_create, which run before any CUDA call."""
import ctypes

import numpy as np
import pytest


def test_weight_file_round_trip_rounds_to_bf16(ngb, tmp_path):
    import torch
    L = ngb.lib()
    n = int(L.ngb_unet_weight_count())
    assert n == sum(cout * 27 * cin for cin, cout in [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (96, 32),
                                                       (32, 32), (48, 16), (16, 16)])
    g = torch.Generator().manual_seed(3)
    w = torch.randn(n, generator=g) * 0.1
    path = str(tmp_path / "w.ngbw")
    assert L.ngb_unet_write_weights(path.encode(), ctypes.c_void_p(w.data_ptr()), n) == 0
    back = torch.empty(n)
    assert L.ngb_unet_read_weights(path.encode(), ctypes.c_void_p(back.data_ptr()), n) == 0
    assert torch.equal(back, w.to(torch.bfloat16).float())  # nearest-even BF16, as torch rounds


def test_weight_file_rejects_other_files(ngb, tmp_path):
    L = ngb.lib()
    n = int(L.ngb_unet_weight_count())
    buf = np.zeros(n, np.float32)
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not a weight file")
    assert L.ngb_unet_read_weights(str(bad).encode(), buf.ctypes.data_as(ctypes.c_void_p), n) == -1
    assert b"not a U-Net weight file" in L.ngb_last_error()
    assert L.ngb_unet_read_weights(str(bad).encode(), buf.ctypes.data_as(ctypes.c_void_p), n - 1) == -1
    assert b"weight count" in L.ngb_last_error()


@pytest.mark.parametrize("n,levels,msg", [(99, 1, b"multiple of 2^levels"), (64, 0, b"levels must be"),
                                           (64, 4, b"coarsest grid"), (36, 1, b"coarsest grid")])
def test_create_rejects_bad_sizes(ngb, n, levels, msg):
    L = ngb.lib()
    w = np.zeros(int(L.ngb_unet_weight_count()), np.float32)
    h = ctypes.c_void_p()
    assert L.ngb_learned_create(n, levels, w.ctypes.data_as(ctypes.c_void_p), w.size, ctypes.byref(h)) == -1
    assert msg in L.ngb_last_error()
    assert not h.value


def test_create_without_network_checks_the_count(ngb):
    """weights NULL means the cycle without the network and needs count 0; a
    weight array needs the full count."""
    L = ngb.lib()
    h = ctypes.c_void_p()
    assert L.ngb_learned_create(64, 1, None, 5, ctypes.byref(h)) == -1
    assert b"weight count" in L.ngb_last_error() and not h.value
    w = np.zeros(4, np.float32)
    assert L.ngb_learned_create(64, 1, w.ctypes.data_as(ctypes.c_void_p), 0, ctypes.byref(h)) == -1
    assert not h.value
