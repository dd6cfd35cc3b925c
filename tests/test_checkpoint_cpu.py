"""Checkpoint files of the dense LBM populations: the loader rejects files that
are not checkpoints, and checkpoints of another lattice, before any CUDA call."""
import struct

import pytest


def _header(nx, ny, nz, q, storage, stride, step=7, omega=1.2, payload=None):
    esz = {0: 8, 1: 4, 2: 2, 3: 2}[storage]
    if payload is None:
        payload = q * stride * esz
    return b"NGBLBM01" + struct.pack("<I5iqqdQ", 1, nx, ny, nz, q, storage, stride, step, omega, payload)


def test_load_rejects_foreign_files(ngb, tmp_path):
    d = ngb.lbm_dense_desc(8, 8, 8, 19, "f32", 1.0)
    p = tmp_path / "x.bin"
    p.write_bytes(b"garbage" * 20)
    with pytest.raises(ngb.NeonError, match="not a population checkpoint"):
        ngb.lbm_dense_load(p, d, 0x1000, None)


def test_load_rejects_other_lattices(ngb, tmp_path):
    d = ngb.lbm_dense_desc(8, 8, 8, 19, "f32", 1.0)
    p = tmp_path / "other.ngbl"
    p.write_bytes(_header(8, 8, 9, 19, 1, 8 * 8 * 9))
    with pytest.raises(ngb.NeonError, match="holds a 8x8x9 D3Q19 lattice"):
        ngb.lbm_dense_load(p, d, 0x1000, None)
    p.write_bytes(_header(8, 8, 8, 19, 2, 512))
    with pytest.raises(ngb.NeonError, match="storage 2"):
        ngb.lbm_dense_load(p, d, 0x1000, None)
    p.write_bytes(_header(8, 8, 8, 19, 1, 512, payload=5))
    with pytest.raises(ngb.NeonError, match="payload of 5 bytes"):
        ngb.lbm_dense_load(p, d, 0x1000, None)


def test_header_layout_is_64_bytes():
    assert len(_header(1, 1, 1, 19, 1, 1)) == 8 + 4 + 20 + 8 + 8 + 8 + 8
