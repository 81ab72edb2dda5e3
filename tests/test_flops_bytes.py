"""The shared work conventions (tenetgb.flops_bytes) against hand counts."""

import pytest


def test_conventions():
    from tenetgb import flops_bytes as F

    assert F.gemm(2, 3, 4) == 8 * 24
    assert F.qr(512, 256, form_q=False) == pytest.approx(4 * (2 * 512 * 256**2 - 2 * 256**3 / 3))
    assert F.qr(256, 512) == F.qr(512, 256)
    assert F.svd(512, 512) == pytest.approx(4 * (4 + 8 + 9) * 512**3)
    assert F.permute_bytes(10, 16) == 320
    assert F.split_gemm_tensor_flops(1, 1, 1, planes=8) == 36 * 8


def test_saturated_tebd_gate_is_13_gflop():
    """χ = 256: 2 QR moves ≈ 1.43 GFLOP, θ 0.54, gate 0.008, SVD 512×512 ≈ 11.3 → ≈ 13.3."""
    from tenetgb import flops_bytes as F

    g = F.tebd_gate(256, 256, 256)
    assert 13.0e9 < g < 13.6e9
    bonds = [2, 4, 8] + [16] * 5 + [8, 4, 2]  # L = 12
    b = [1] + bonds + [1]
    assert F.tebd_layer(bonds, 2, 5) == pytest.approx(sum(F.tebd_gate(b[a - 1], b[a], b[a + 1]) for a in (2, 4, 6, 8, 10)))


def test_canonize_compress_matches_a_hand_sweep():
    from tenetgb import flops_bytes as F

    # L = 3, d = 2, bonds (2, 2), maxdim 1
    tot = F.canonize_compress(3, [2, 2], 1)
    qr_part = F.qr(2, 2) + F.gemm(2, 4, 2) + F.qr(4, 2) + F.gemm(2, 2, 2)
    lq_part = F.qr(2, 2) + F.gemm(4, 2, 2) + F.qr(4, 2) + F.gemm(2, 2, 2)
    svd_part = F.svd(2, 2) + F.gemm(1, 2, 2) + F.gemm(1, 4, 2) + F.svd(2, 2) + F.gemm(1, 2, 2) + F.gemm(1, 2, 2)
    assert tot == pytest.approx(qr_part + lq_part + svd_part)
