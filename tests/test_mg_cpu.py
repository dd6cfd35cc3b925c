"""Host logic of the multilevel learned preconditioner (no GPU): level
descriptors, buffer sizes and argument checks of VCycle."""
import pytest


def test_vcycle_levels_and_buffers():
    torch = pytest.importorskip("torch")
    from neon_gb300 import fcg
    vc = fcg.VCycle(64, 2, coarse="none", device="cpu")
    assert [(d.nx, d.h) for d in vc.descs] == [(64, 1.0), (32, 2.0), (16, 4.0)]
    assert [t.numel() for t in vc.u] == [64 ** 3, 32 ** 3]
    assert vc.r[0] is None and [t.numel() for t in vc.r[1:]] == [32 ** 3, 16 ** 3]
    assert float(vc.coarse_mask.sum()) == 14 ** 3


def test_vcycle_rejects_bad_shapes():
    pytest.importorskip("torch")
    from neon_gb300 import fcg
    with pytest.raises(ValueError):
        fcg.VCycle(96, 4, coarse="none", device="cpu")  # 96 / 16 = 6 < 8 nodes on the coarsest level
    with pytest.raises(ValueError):
        fcg.VCycle(100, 3, coarse="none", device="cpu")  # not divisible by 8
    with pytest.raises(ValueError):
        fcg.VCycle(64, 2, net=None, coarse="net", device="cpu")
    with pytest.raises(ValueError):
        fcg.VCycle(64, 2, coarse="multigrid", device="cpu")
