"""GPU checks of the learned preconditioner's kernels against the numpy oracle
(oracle/unet_oracle.py): tensor-core convolution forward / backward-data /
backward-weight, pooling, upsampling, the whole U-Net forward pass and its
gradients."""
import ctypes

import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


def _bf16_tensor(a, dev):
    import torch
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).to(dev)


@pytest.mark.parametrize("cin,cout", [(16, 16), (32, 64), (96, 32), (48, 16), (16, 8)])
def test_conv_forward_matches_oracle(ngb, cuda, cin, cout):
    import torch
    rng = np.random.default_rng(cin * 100 + cout)
    n = (6, 5, 7)  # nz, ny, nx
    x = U.bf16(rng.standard_normal(n + (cin,)))
    w = U.bf16(rng.standard_normal((cout, 27, cin)) / np.sqrt(27 * cin))
    ref = U.conv(x, w)
    X = _bf16_tensor(x.reshape(-1, cin), cuda)
    Wt = _bf16_tensor(w, cuda)
    Y = torch.zeros(X.shape[0], cout, dtype=torch.float32, device=cuda)
    ngb.check(ngb.lib().ngb_conv3d(7, 5, 6, ngb._ptr(X), cin, cin, ngb._ptr(Wt), None, ngb._ptr(Y), cout, cout, 1, 0, 0, None))
    got = Y.cpu().numpy().reshape(ref.shape)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    # BF16 output with ReLU
    Yb = torch.zeros(X.shape[0], cout, dtype=torch.bfloat16, device=cuda)
    ngb.check(ngb.lib().ngb_conv3d(7, 5, 6, ngb._ptr(X), cin, cin, ngb._ptr(Wt), None, ngb._ptr(Yb), cout, cout, 0, 1, 0, None))
    gotb = Yb.float().cpu().numpy().reshape(ref.shape)
    assert np.abs(gotb - U.bf16(np.maximum(ref, 0))).max() <= 2 ** -7 * np.abs(ref).max()


@pytest.mark.parametrize("cin,cout", [(16, 16), (48, 16), (32, 64), (96, 32)])
def test_conv_backward_weight_and_data(ngb, cuda, cin, cout):
    import torch
    rng = np.random.default_rng(7 + cin + cout)
    nz, ny, nx = 6, 8, 5
    x = U.bf16(rng.standard_normal((nz, ny, nx, cin)))
    dy = U.bf16(rng.standard_normal((nz, ny, nx, cout)))
    w = U.bf16(rng.standard_normal((cout, 27, cin)) / np.sqrt(27 * cin))
    dw_ref = U.conv_bwd_weight(x, dy)
    dx_ref = U.conv_bwd_data(dy, w)
    X = _bf16_tensor(x.reshape(-1, cin), cuda)
    D = _bf16_tensor(dy.reshape(-1, cout), cuda)
    dW = torch.zeros(cout, 27, cin, dtype=torch.float32, device=cuda)
    L = ngb.lib()
    ngb.check(L.ngb_conv3d_bwd_weight(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dW), None))
    assert np.abs(dW.cpu().numpy() - dw_ref).max() <= 1e-5 * np.abs(dw_ref).max()
    Wf = torch.from_numpy(w.astype(np.float32)).to(cuda)
    Wt = torch.empty(cin, 27, cout, dtype=torch.bfloat16, device=cuda)
    ngb.check(L.ngb_flip_weights(cout, cin, ngb._ptr(Wf), ngb._ptr(Wt), None))
    dX = torch.zeros(X.shape[0], cin, dtype=torch.float32, device=cuda)
    if cin <= 64:
        ngb.check(L.ngb_conv3d(nx, ny, nz, ngb._ptr(D), cout, cout, ngb._ptr(Wt), None, ngb._ptr(dX), cin, cin, 1, 0, 0, None))
    else:  # 96 output channels in two calls of 64 and 32 (the U-Net's c1c)
        for lo, hi in ((0, 64), (64, 96)):
            ptr = ctypes.c_void_p(dX.data_ptr() + lo * 4)
            ngb.check(L.ngb_conv3d(nx, ny, nz, ngb._ptr(D), cout, cout, ngb._ptr(Wt[lo:hi]), None, ptr, cin, hi - lo, 1, 0, 0,
                                   None))
    assert np.abs(dX.cpu().numpy().reshape(dx_ref.shape) - dx_ref).max() <= 1e-5 * np.abs(dx_ref).max()


def test_pool_and_upsample(ngb, cuda):
    import torch
    rng = np.random.default_rng(5)
    x = U.bf16(rng.standard_normal((4, 6, 8, 16)))
    X = _bf16_tensor(x.reshape(-1, 16), cuda)
    P = torch.zeros(2 * 3 * 4, 16, dtype=torch.bfloat16, device=cuda)
    L = ngb.lib()
    ngb.check(L.ngb_pool2(8, 6, 4, 16, ngb._ptr(X), 16, ngb._ptr(P), 16, None))
    assert np.allclose(P.float().cpu().numpy().reshape(2, 3, 4, 16), U.bf16(U.pool(x)), rtol=0, atol=1e-6)
    Up = torch.zeros_like(X)
    ngb.check(L.ngb_up2(8, 6, 4, 16, ngb._ptr(P), 16, ngb._ptr(Up), 16, None))
    assert np.array_equal(Up.float().cpu().numpy().reshape(x.shape), U.up(P.float().cpu().numpy().reshape(2, 3, 4, 16)))


@pytest.mark.parametrize("C,ld,off", [(32, 48, 16), (16, 48, 32), (12, 20, 4), (8, 8, 0)])
def test_pool_and_upsample_channel_ranges(ngb, cuda, C, ld, off):
    """Pooling and upsampling on a channel range of wider channels-last
    buffers: 16-byte vector kernels where the range and strides allow
    (multiples of 8 channels, 16-byte aligned), the per-channel kernels
    otherwise; elements outside the range untouched."""
    import torch
    rng = np.random.default_rng(C + ld + off)
    nz, ny, nx = 6, 4, 10
    x = U.bf16(rng.standard_normal((nz, ny, nx, C)))
    X = torch.zeros(nx * ny * nz, ld, dtype=torch.bfloat16, device=cuda)
    X[:, off:off + C] = _bf16_tensor(x.reshape(-1, C), cuda)
    P = torch.full((nx * ny * nz // 8, ld), 7.0, dtype=torch.bfloat16, device=cuda)
    L = ngb.lib()
    pX = ctypes.c_void_p(X.data_ptr() + 2 * off)
    pP = ctypes.c_void_p(P.data_ptr() + 2 * off)
    ngb.check(L.ngb_pool2(nx, ny, nz, C, pX, ld, pP, ld, None))
    got = P[:, off:off + C].float().cpu().numpy().reshape(nz // 2, ny // 2, nx // 2, C)
    assert np.allclose(got, U.bf16(U.pool(x)), rtol=0, atol=1e-6)
    assert float(P[:, :off].float().sub(7.0).abs().max() if off else 0.0) == 0.0
    Up = torch.full_like(X, 5.0)
    pU = ctypes.c_void_p(Up.data_ptr() + 2 * off)
    ngb.check(L.ngb_up2(nx, ny, nz, C, pP, ld, pU, ld, None))
    assert np.array_equal(Up[:, off:off + C].float().cpu().numpy().reshape(x.shape), U.up(got))
    rest = torch.cat([Up[:, :off], Up[:, off + C:]], 1)
    assert rest.numel() == 0 or float((rest.float() - 5.0).abs().max()) == 0.0


def test_unet_forward_and_gradients_match_oracle(ngb, cuda):
    import torch
    from neon_gb300.learned import UNet
    n = 12
    net = UNet(seed=4, device=cuda)
    # non-trivial last layer so gradients reach every layer
    net.w["c0d"] = net.w["c0d"] * 0 + torch.randn(net.w["c0d"].shape, generator=torch.Generator().manual_seed(9)).to(cuda) * 0.05
    net.load_state_dict({k: v.cpu() for k, v in net.w.items()})
    rng = np.random.default_rng(11)
    r = rng.standard_normal(n ** 3).astype(np.float32)
    e = rng.standard_normal(n ** 3).astype(np.float32)
    z = net.forward(torch.from_numpy(r).to(cuda))
    W = {k: v.cpu().numpy().astype(np.float64) for k, v in net.w.items()}
    zo, cache = U.forward(W, r, n)
    zg = z.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(zg - zo) <= 2e-3 * np.linalg.norm(zo), np.linalg.norm(zg - zo) / np.linalg.norm(zo)
    dz = (zg - e).astype(np.float32)
    net.zero_grad()
    net.backward(torch.from_numpy(dz).to(cuda))
    go = U.backward(cache, dz.astype(np.float64))
    for name in go:
        gg = net.g[name].cpu().numpy()
        rel = np.linalg.norm(gg - go[name]) / max(np.linalg.norm(go[name]), 1e-30)
        assert rel <= 2e-2, (name, rel)


def test_training_reduces_loss(ngb, cuda):
    import torch
    from neon_gb300.learned import UNet
    n = 16
    net = UNet(seed=1, device=cuda)
    g = torch.Generator().manual_seed(2)
    r = torch.randn(n ** 3, generator=g).to(cuda)
    target = torch.roll(r, 1) * 0.5 + r  # a fixed linear map of r
    losses = []
    for it in range(60):
        z = net.forward(r)
        diff = z - target
        losses.append(float((diff ** 2).sum() / (target ** 2).sum()))
        net.zero_grad()
        net.backward(2 * diff / (target ** 2).sum())
        net.adam_step(lr=3e-3)
    assert losses[-1] < 0.5 * losses[0], losses[::10]


@pytest.mark.parametrize("dims", [(3, 4, 32), (2, 3, 128), (2, 2, 256)])
@pytest.mark.parametrize("cin,cout", [(16, 16), (32, 64), (96, 32), (48, 16), (16, 48), (32, 96), (64, 64)])
def test_conv_tensor_cores_match_oracle(ngb, cuda, dims, cin, cout):
    """tcgen05 convolution (TMA-staged operands, TMEM accumulators) against the
    float64 oracle on the same BF16 inputs: FP32 output with and without
    accumulation, BF16 output with ReLU; tile edges at the x, y and z faces."""
    import torch
    nz, ny, nx = dims
    L = ngb.lib()
    assert L.ngb_conv3d_tc_supported(nx, ny, nz, cin, cin, cout, cout) == 1
    rng = np.random.default_rng(cin * 1000 + cout + nx)
    x = U.bf16(rng.standard_normal((nz, ny, nx, cin)))
    w = U.bf16(rng.standard_normal((cout, 27, cin)) / np.sqrt(27 * cin))
    ref = U.conv(x, w)
    X = _bf16_tensor(x.reshape(-1, cin), cuda)
    Wt = _bf16_tensor(w, cuda)
    Wp = torch.empty_like(Wt)
    ngb.check(L.ngb_conv3d_pack(cout, cin, ngb._ptr(Wt), ngb._ptr(Wp), None))
    Y = torch.zeros(X.shape[0], cout, dtype=torch.float32, device=cuda)
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), None, ngb._ptr(Y), cout, cout, 1, 0, 0, None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    got = Y.cpu().numpy().reshape(ref.shape)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-5 * scale, np.abs(got - ref).max() / scale
    # accumulate into the existing FP32 output: 2 x ref
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), None, ngb._ptr(Y), cout, cout, 1, 0, 1, None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    assert np.abs(Y.cpu().numpy().reshape(ref.shape) - 2 * ref).max() <= 2e-5 * scale
    # BF16 output with ReLU, written into a channel range of a wider buffer
    wide = cout + 16
    Yb = torch.zeros(X.shape[0], wide, dtype=torch.bfloat16, device=cuda)
    ptr = ctypes.c_void_p(Yb.data_ptr() + 16 * 2)
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), None, ptr, wide, cout, 0, 1, 0, None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    gotb = Yb[:, 16:].float().cpu().numpy().reshape(ref.shape)
    assert np.abs(gotb - U.bf16(np.maximum(ref, 0))).max() <= 2 ** -7 * scale
    assert float(Yb[:, :16].abs().max()) == 0.0


def test_conv_tensor_cores_reject_unsupported_shapes(ngb):
    L = ngb.lib()
    assert L.ngb_conv3d_tc_supported(12, 12, 12, 16, 16, 16, 16) == 0  # 12 does not divide 128
    assert L.ngb_conv3d_tc_supported(32, 6, 4, 16, 16, 16, 16) == 0  # 128 / 32 rows do not tile ny = 6
    assert L.ngb_conv3d_tc_supported(128, 1, 1, 16, 16, 8, 8) == 0  # cout 8 (N must be a multiple of 16)
    assert L.ngb_conv3d_tc_supported(128, 1, 1, 16, 16, 16, 16) == 1
    rc = L.ngb_conv3d_tc(12, 12, 12, None, 16, 16, None, None, None, 16, 16, 0, 0, 0, None)
    assert rc != 0


def test_unet_tensor_cores_match_oracle_and_mma_path(ngb, cuda):
    """At 32^3 levels 0 and 1 run on tcgen05 (level 2, 8^3, on mma.sync): the
    forward pass and all gradients against the numpy oracle, and the forward
    pass against the all-mma.sync network."""
    import torch
    from neon_gb300.learned import UNet
    n = 32
    net = UNet(seed=4, device=cuda)
    net.w["c0d"] = net.w["c0d"] * 0 + torch.randn(net.w["c0d"].shape, generator=torch.Generator().manual_seed(9)).to(cuda) * 0.05
    net.load_state_dict({k: v.cpu() for k, v in net.w.items()})
    rng = np.random.default_rng(12)
    r = rng.standard_normal(n ** 3).astype(np.float32)
    e = rng.standard_normal(n ** 3).astype(np.float32)
    z = net.forward(torch.from_numpy(r).to(cuda)).clone()
    W = {k: v.cpu().numpy().astype(np.float64) for k, v in net.w.items()}
    zo, cache = U.forward(W, r, n)
    zg = z.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(zg - zo) <= 2e-3 * np.linalg.norm(zo), np.linalg.norm(zg - zo) / np.linalg.norm(zo)
    dz = (zg - e).astype(np.float32)
    net.zero_grad()
    net.backward(torch.from_numpy(dz).to(cuda))
    go = U.backward(cache, dz.astype(np.float64))
    for name in go:
        gg = net.g[name].cpu().numpy()
        rel = np.linalg.norm(gg - go[name]) / max(np.linalg.norm(go[name]), 1e-30)
        assert rel <= 2e-2, (name, rel)
    net.tensor_cores = False
    z2 = net.forward(torch.from_numpy(r).to(cuda)).clone()
    assert float((z - z2).norm() / z2.norm()) <= 2e-3


@pytest.mark.parametrize("dims", [(8, 64, 128), (4, 32, 256), (16, 64, 64), (7, 33, 128)])
@pytest.mark.parametrize("cin,cout", [(16, 16), (48, 16), (32, 96), (64, 64)])
def test_conv_tensor_cores_many_tiles_match_mma(ngb, cuda, dims, cin, cout):
    """Grids with many more tiles than resident CTAs, so each persistent CTA
    cycles through both TMEM accumulator buffers and many barrier phases:
    the tcgen05 convolution against the mma.sync kernel on the same inputs
    (plane mode, tap mode, and an odd ny that falls back to one-tile units)."""
    import torch
    nz, ny, nx = dims
    L = ngb.lib()
    assert L.ngb_conv3d_tc_supported(nx, ny, nz, cin, cin, cout, cout) == 1
    g = torch.Generator(device="cpu").manual_seed(cin + cout + nx + ny)
    X = torch.randn(nx * ny * nz, cin, generator=g).to(torch.bfloat16).to(cuda)
    W = (torch.randn(cout, 27, cin, generator=g) / (27 * cin) ** 0.5).to(torch.bfloat16).to(cuda)
    Wp = torch.empty_like(W)
    ngb.check(L.ngb_conv3d_pack(cout, cin, ngb._ptr(W), ngb._ptr(Wp), None))
    ref = torch.zeros(X.shape[0], cout, dtype=torch.float32, device=cuda)
    for lo in range(0, cout, 64):
        hi = min(cout, lo + 64)
        ptr = ctypes.c_void_p(ref.data_ptr() + lo * 4)
        ngb.check(L.ngb_conv3d(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(W[lo:hi]), None, ptr, cout, hi - lo, 1, 0, 0, None))
    Y = torch.full_like(ref, float("nan"))
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), None, ngb._ptr(Y), cout, cout, 1, 0, 0, None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    scale = float(ref.abs().max())
    err = float((Y - ref).abs().max())
    assert err <= 1e-5 * scale, (err / scale, int(torch.isnan(Y).sum()))


@pytest.mark.parametrize("dims", [(79, 128, 512), (37, 4, 128), (3, 2, 128), (20, 8, 64), (9, 3, 128), (64, 64, 64)])
@pytest.mark.parametrize("cin,cout", [(16, 16), (48, 16), (16, 32), (32, 32), (96, 32)])
def test_conv_tensor_cores_z_runs_match_mma(ngb, cuda, dims, cin, cout):
    """Layers with Cout 16 / 32 and resident weights (plane mode, 96 -> 32 with
    162 KB of weights at one CTA per SM; tap mode for rows of 64 voxels or an
    odd row count) march each work unit over a run of output planes (16 at the largest size here, 4 on the small grids; the
    last run ragged, a grid shorter than one run): every input plane staged
    once, the three output planes it feeds accumulated in a ring of TMEM
    slots. Against the mma.sync kernel, FP32 output with bias and with
    accumulation, BF16 output with ReLU."""
    import torch
    nz, ny, nx = dims
    L = ngb.lib()
    assert L.ngb_conv3d_tc_supported(nx, ny, nz, cin, cin, cout, cout) == 1
    g = torch.Generator(device="cpu").manual_seed(7 * cin + cout + nz)
    X = torch.randn(nx * ny * nz, cin, generator=g).to(torch.bfloat16).to(cuda)
    W = (torch.randn(cout, 27, cin, generator=g) / (27 * cin) ** 0.5).to(torch.bfloat16).to(cuda)
    bias = torch.randn(cout, generator=g).to(cuda) * 0.1
    Wp = torch.empty_like(W)
    ngb.check(L.ngb_conv3d_pack(cout, cin, ngb._ptr(W), ngb._ptr(Wp), None))
    ref = torch.zeros(X.shape[0], cout, dtype=torch.float32, device=cuda)
    ngb.check(L.ngb_conv3d(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(W), None, ngb._ptr(ref), cout, cout, 1, 0, 0, None))
    ref += bias
    Y = torch.full_like(ref, float("nan"))
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), ngb._ptr(bias), ngb._ptr(Y), cout, cout, 1, 0, 0,
                              None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    scale = float(ref.abs().max())
    assert float((Y - ref).abs().max()) <= 1e-5 * scale, int(torch.isnan(Y).sum())
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), ngb._ptr(bias), ngb._ptr(Y), cout, cout, 1, 0, 1,
                              None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    assert float((Y - 2 * ref).abs().max()) <= 2e-5 * scale
    Yb = torch.zeros(X.shape[0], cout, dtype=torch.bfloat16, device=cuda)
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), ngb._ptr(bias), ngb._ptr(Yb), cout, cout, 0, 1, 0,
                              None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    assert float((Yb.float() - ref.clamp(min=0)).abs().max()) <= 2 ** -7 * scale


def test_unet_tensor_cores_match_mma_path_at_128(ngb, cuda):
    """At 128^3 level 0 runs in plane mode with many tiles per CTA: the U-Net
    forward pass and the layer gradients on the tensor cores against the
    mma.sync network."""
    import torch
    from neon_gb300.learned import UNet
    n = 128
    net = UNet(seed=5, device=cuda)
    net.w["c0d"] = net.w["c0d"] * 0 + torch.randn(net.w["c0d"].shape, generator=torch.Generator().manual_seed(3)).to(cuda) * 0.05
    net.load_state_dict({k: v.cpu() for k, v in net.w.items()})
    g = torch.Generator(device="cpu").manual_seed(21)
    r = torch.randn(n ** 3, generator=g).to(cuda)
    e = torch.randn(n ** 3, generator=g).to(cuda)
    out = {}
    for tc in (True, False):
        net.tensor_cores = tc
        z = net.forward(r).clone()
        net.zero_grad()
        net.backward(z - e)
        out[tc] = (z, {k: v.clone() for k, v in net.g.items()})
    (z1, g1), (z0, g0) = out[True], out[False]
    assert torch.isfinite(z1).all()
    assert float((z1 - z0).norm() / z0.norm()) <= 2e-3
    for name in g0:
        rel = float((g1[name] - g0[name]).norm() / max(float(g0[name].norm()), 1e-30))
        assert rel <= 2e-2, (name, rel)


def test_bounded_wait_times_out_and_reports(ngb, cuda):
    """A bounded mbarrier wait on a barrier nothing arrives on (no copy or MMA
    in flight) gives up after its limit; the flag it raises is what
    ngb_conv3d_tc_check reports as NGB_ERR_TIMEOUT, once, and the context
    stays usable (a convolution afterwards still checks clean)."""
    import torch
    L = ngb.lib()
    assert L.ngb_conv3d_tc_wait_selftest(4096, None) == 0, L.ngb_last_error()
    assert L.ngb_conv3d_tc_check(None) == -5  # NGB_ERR_TIMEOUT
    assert b"wait ran out" in L.ngb_last_error()
    assert L.ngb_conv3d_tc_check(None) == 0  # the flag was cleared
    assert L.ngb_conv3d_tc_wait_selftest(0, None) == -1  # limit out of range
    nx, ny, nz = 16, 8, 4
    cin = cout = 16
    assert L.ngb_conv3d_tc_supported(nx, ny, nz, cin, cin, cout, cout) == 1
    X = torch.randn(nx * ny * nz, cin, device=cuda).to(torch.bfloat16)
    W = (torch.randn(cout, 27, cin, device=cuda) * 0.05).to(torch.bfloat16)
    Wp = torch.empty_like(W)
    ngb.check(L.ngb_conv3d_pack(cout, cin, ngb._ptr(W), ngb._ptr(Wp), None))
    Y = torch.zeros(nx * ny * nz, cout, dtype=torch.float32, device=cuda)
    ngb.check(L.ngb_conv3d_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(Wp), None, ngb._ptr(Y), cout, cout, 1, 0, 0, None))
    ngb.check(L.ngb_conv3d_tc_check(None))
    assert bool(torch.isfinite(Y).all())


@pytest.mark.parametrize("dims,cin,cout", [((8, 8, 8), 16, 16), ((16, 8, 8), 32, 64), ((8, 16, 8), 48, 16), ((8, 8, 16), 64, 64),
                                           ((16, 8, 8), 96, 32), ((24, 8, 8), 16, 32)])
def test_conv_backward_weight_tensor_cores_match_oracle(ngb, cuda, dims, cin, cout):
    """The tcgen05 weight gradient (tap groups of 128 / cin rows, K = voxels,
    operands transposed into shared memory) against the float64 oracle on
    shapes it takes, every tap group (partial last groups, padded rows for
    cin = 48 and 96) and several CTAs per group; BF16 products are exact in
    FP32, so only the summation order differs: within 1e-5 of the largest
    entry. The mma.sync form on the same input agrees as well."""
    import torch
    nx, ny, nz = dims
    rng = np.random.default_rng(nx * 7 + cin + cout)
    x = U.bf16(rng.standard_normal((nz, ny, nx, cin)))
    dy = U.bf16(rng.standard_normal((nz, ny, nx, cout)))
    dw_ref = U.conv_bwd_weight(x, dy)
    X = _bf16_tensor(x.reshape(-1, cin), cuda)
    D = _bf16_tensor(dy.reshape(-1, cout), cuda)
    L = ngb.lib()
    assert L.ngb_conv3d_bwd_weight_tc_supported(nx, ny, nz, cin, cin, cout, cout) == 1
    dW = torch.zeros(cout, 27, cin, dtype=torch.float32, device=cuda)
    ngb.check(L.ngb_conv3d_bwd_weight_tc(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dW), None))
    scale = np.abs(dw_ref).max()
    assert np.abs(dW.cpu().numpy() - dw_ref).max() <= 1e-5 * scale
    dM = torch.zeros_like(dW)
    ngb.check(L.ngb_conv3d_bwd_weight_mma(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dM), None))
    assert float((dW - dM).abs().max()) <= 1e-5 * scale
    # accumulation into dw (the training path adds the gradients of a batch)
    ngb.check(L.ngb_conv3d_bwd_weight(nx, ny, nz, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dW), None))
    assert np.abs(dW.cpu().numpy() - 2 * dw_ref).max() <= 2e-5 * scale


def test_conv_backward_weight_tensor_cores_at_64(ngb, cuda):
    """Level-0 shape of training at 64^3 (cin 16, cout 16; 262144 voxels,
    many CTAs per tap group adding into dw): tcgen05 against mma.sync."""
    import torch
    n, cin, cout = 64, 16, 16
    g = torch.Generator(device="cpu").manual_seed(5)
    X = torch.randn(n ** 3, cin, generator=g).to(torch.bfloat16).to(cuda)
    D = torch.randn(n ** 3, cout, generator=g).to(torch.bfloat16).to(cuda)
    L = ngb.lib()
    dW = torch.zeros(cout, 27, cin, dtype=torch.float32, device=cuda)
    dM = torch.zeros_like(dW)
    ngb.check(L.ngb_conv3d_bwd_weight_tc(n, n, n, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dW), None))
    ngb.check(L.ngb_conv3d_bwd_weight_mma(n, n, n, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dM), None))
    scale = float(dM.abs().max())
    assert float((dW - dM).abs().max()) <= 1e-4 * scale


def test_conv_backward_weight_tensor_cores_are_deterministic(ngb, cuda):
    """The CTAs' partial sums meet in a fixed order: repeated calls give the
    same bits (training runs repeat exactly)."""
    import torch
    n, cin, cout = 32, 16, 32
    g = torch.Generator(device="cpu").manual_seed(11)
    X = torch.randn(n ** 3, cin, generator=g).to(torch.bfloat16).to(cuda)
    D = torch.randn(n ** 3, cout, generator=g).to(torch.bfloat16).to(cuda)
    L = ngb.lib()
    outs = []
    for _ in range(3):
        dW = torch.zeros(cout, 27, cin, dtype=torch.float32, device=cuda)
        ngb.check(L.ngb_conv3d_bwd_weight_tc(n, n, n, ngb._ptr(X), cin, cin, ngb._ptr(D), cout, cout, ngb._ptr(dW), None))
        outs.append(dW.cpu().numpy().view(np.uint32))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
