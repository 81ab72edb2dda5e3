"""Dump / load of device MPS (tn_mps_save / tn_mps_load): every instance, the bond
dimensions, the canonical form and Λ come back bit for bit; a loaded MPS serves queries."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rand_sites(rng, bonds, d=2):
    return [(rng.standard_normal((bonds[i], d, bonds[i + 1])) + 1j * rng.standard_normal((bonds[i], d, bonds[i + 1])))
            for i in range(len(bonds) - 1)]


def test_save_load_round_trip(tmp_path):
    import tenetgb

    rng = np.random.default_rng(61)
    bonds = [1, 2, 4, 8, 4, 2, 1]
    psi = tenetgb.MPS.batched([rand_sites(rng, bonds) for _ in range(3)], max_bond=16)
    psi.canonize_(tenetgb.BondCanonical(3, 4))
    path = tmp_path / "psi.tnmps"
    psi.save(path)
    phi = tenetgb.MPS.load(path, max_bond=16)
    assert phi.batch == 3 and phi.nsites == 6
    assert phi.bondsizes() == psi.bondsizes()
    f = phi.form
    assert isinstance(f, tenetgb.BondCanonical) and (f.a, f.b) == (3, 4)
    np.testing.assert_array_equal(phi.lambda_(), psi.lambda_())
    for b in range(3):
        for i in range(1, 7):
            np.testing.assert_array_equal(phi.site(i, b), psi.site(i, b))
    # the loaded MPS is a working MPS
    np.testing.assert_allclose(phi.norm(), psi.norm(), rtol=1e-14)


def test_load_rejects_other_files(tmp_path):
    import tenetgb

    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not an mps dump at all")
    with pytest.raises(ValueError):
        tenetgb.MPS.load(bad)
    with pytest.raises(ValueError):
        tenetgb.MPS.load(tmp_path / "missing.bin")
