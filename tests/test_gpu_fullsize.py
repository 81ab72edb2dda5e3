"""Parity at the full benchmark sizes, through the C ABI.

* TEBD χ=256 (L=64, d=2, χ0=16, ten brickwork layers of seeded Haar gates, maxdim 256,
  absolute cutoff 1e-12): the plain FP64 GPU path against the oracle after every
  layer — ⟨ψ|ψ⟩ to ≤ 1e-12 relative, ⟨Z_i⟩ to ≤ 1e-12, identical bond dimensions — with
  the relative gap (σ_χ − σ_χ+1)/σ_χ at every truncated cut reported beside the error.
  The same run repeated in the oracle with LAPACK's QR-iteration SVD (gesvd instead of
  gesdd) measures how far rounding alone moves the truncated state.
* One saturated gate (θ 512×512, layer 6 on bond 32-33 of that state) at the Muscle
  level (tn_simple_update) on identical inputs: kept rank equal, kept singular values to
  ≤ 1e-12 of σ_max, reconstructed θ' = A'·B' to ≤ 1e-12 relative; for the plain FP64,
  mixed and split-BF16 forms.
* The closed 8×8 lattice (bond 8, seed 4) contracted to a scalar along the greedy path:
  FP64 GPU against the complex128 oracle along the same path to ≤ 1e-12.
* The 512-MPS ragged population (canonize → compress(χ/2) → norm, one grouped call):
  norms against the oracle and the per-instance device path.

These take minutes of oracle time on the host cores (marked slow as well as gpu).
"""

import json
import os

import numpy as np
import pytest

from oracle import network_oracle as NO
from oracle import tenet_oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

L_SITES, CHI, CUT = 64, 256, 1e-12


@pytest.fixture(scope="module")
def ctx():
    import tenetgb

    return tenetgb.Context(0)


@pytest.fixture(scope="module")
def tebd_run(ctx):
    """Device FP64 and oracle (gesdd, gesvd) over the ten layers, one layer at a time."""
    import tenetgb
    from tenetgb import workloads as W

    sites, layers = W.tebd_workload(L=L_SITES, chi0=16, n_layers=10)
    Z = W.pauli_z()
    psi = tenetgb.MPS(sites, ctx=ctx, max_bond=CHI, precision="native")
    p_dd = O.OMPS([s.copy() for s in sites])
    p_dv = O.OMPS([s.copy() for s in sites])
    rows, sat = [], None
    for ell, ly in enumerate(layers):
        psi.evolve_brickwork_([ly], maxdim=CHI, threshold=CUT)
        spectra = []
        O.tebd(p_dd, [ly], CHI, CUT, spectra=spectra)
        O.tebd(p_dv, [ly], CHI, CUT, driver="gesvd")
        ov, ov_dd, ov_dv = psi.overlap(psi), O.overlap(p_dd, p_dd), O.overlap(p_dv, p_dv)
        z = psi.local_expectations(Z)
        z_dd, _ = O.local_expectations(p_dd, Z)
        z_dv, _ = O.local_expectations(p_dv, Z)
        gaps = [g for g in (O.truncation_gap(s, CHI, CUT) for s in spectra) if np.isfinite(g)]
        rows.append(dict(layer=ell + 1, bonds_equal=psi.bondsizes() == p_dd.bondsizes(),
                         overlap_gpu_vs_oracle=abs(ov - ov_dd) / abs(ov_dd),
                         overlap_gesvd_vs_gesdd=abs(ov_dv - ov_dd) / abs(ov_dd),
                         z_gpu_vs_oracle=float(np.abs(z - z_dd).max()),
                         z_gesvd_vs_gesdd=float(np.abs(z_dv - z_dd).max()),
                         truncated_cuts=len(gaps), min_relative_gap=min(gaps) if gaps else None))
        if ell == 4:
            sat = [psi.site(i) for i in range(1, L_SITES + 1)]
    print("\n" + "\n".join(json.dumps(r) for r in rows))
    return rows, sat, layers


def test_tebd_chi256_fp64_matches_oracle_every_layer(tebd_run):
    rows, _, _ = tebd_run
    for r in rows:
        assert r["bonds_equal"], r
        assert r["overlap_gpu_vs_oracle"] <= 1e-12, r
        assert r["z_gpu_vs_oracle"] <= 1e-12, r
    # the cap binds from layer 5 on, with the cut inside the spectrum
    assert all(r["truncated_cuts"] > 0 for r in rows[4:])


@pytest.mark.parametrize("precision", ["native", "mixed", "split_bf16"])
def test_saturated_gate_matches_oracle(ctx, tebd_run, precision):
    import tenetgb

    _, sat, layers = tebd_run
    g = tenetgb.MPS(sat, ctx=ctx, max_bond=CHI)
    g.canonize_([32, 33])
    A, B = g.site(32), g.site(33)
    start, gates = layers[5][0], layers[5][1]
    G = gates[(32 - start) // 2]
    An_o, Bn_o, s_kept, s_full = O.simple_update_tensors(A, B, G, CHI, CUT)
    gap = O.truncation_gap(s_full, CHI, CUT)
    th_o = np.tensordot(An_o, Bn_o, axes=(2, 0))
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["l", "a", "m"])
    dB = tenetgb.DeviceTensor.from_numpy(ctx, B, ["m", "b", "r"])
    dG = tenetgb.DeviceTensor.from_numpy(ctx, G, ["ao", "bo", "a", "b"])
    An, Bn = tenetgb.simple_update(dA, "a", dB, "b", "m", dG, "ao", "bo", maxdim=CHI, threshold=CUT,
                                   precision=precision)
    an, bn = An.numpy(), Bn.numpy()
    assert an.shape[2] == s_kept.size == CHI
    # A' = U√S: the squared singular values of A' are the kept values
    s_dev = np.linalg.svd(an.reshape(-1, an.shape[2]), compute_uv=False) ** 2
    s_err = np.abs(np.sort(s_dev)[::-1] - s_kept).max() / s_kept[0]
    th = np.tensordot(an, bn, axes=(2, 0))
    th_err = np.linalg.norm(th - th_o) / np.linalg.norm(th_o)
    print(f"\n{precision}: relative gap at the cut {gap:.3e}; kept S {s_err:.2e}; theta' {th_err:.2e}")
    assert s_err <= 1e-12
    assert th_err <= 1e-12


def test_lattice_8x8_bond8_fp64_matches_oracle(ctx):
    import math

    from tenetgb import network as N

    net = N.lattice_2d(8, 8, 8, seed=4)
    path = N.greedy_path(net.labels, net.dims)
    ref = NO.contract_along(net.arrays, net.labels, path)
    val = N.contract(net, path, precision="native", dtype=np.complex128, ctx=ctx)
    scale = math.prod(float(np.linalg.norm(a)) for a in net.arrays)
    err = abs(val - ref) / abs(ref)
    print(f"\n8x8 lattice: |ref| = {abs(ref):.6e} (product of norms {scale:.3e}); relative error {err:.2e}")
    assert err <= 1e-12


def test_batched_512_population_norms(ctx):
    """Config 4 at its full size: the 512-MPS ragged population (L in [16, 128], χ
    log-uniform in [16, 512], seed 5), canonize → compress(χ/2) → norm in one grouped
    call.  The norms of the 150 cheapest instances (by L·χ³) are checked against the
    oracle on their initial sites to 1e-12 relative, and 12 instances spread over the χ
    range (the largest included) against the per-instance device path to 1e-10: the two
    device paths order their Jacobi rotations differently, so at a cut inside a dense
    random spectrum (512 values, smallest relative gaps ~1e-5) the kept vectors agree to
    ε/gap, and the downstream truncations carry that into the norm."""
    import tenetgb
    from tenetgb import workloads as W
    from tenetgb.group import MPSGroup

    Ls, chis = W.batched_population()
    maxdim = [max(1, c // 2) for c in chis]
    g = MPSGroup.random(Ls, chis, seed=5, ctx=ctx)
    ctx.sync()
    cost = np.array([L * c**3 for L, c in zip(Ls, chis)])
    cheap = list(np.argsort(cost)[:150])
    spread = list(np.argsort(chis)[np.linspace(0, len(chis) - 1, 12).astype(int)])
    init = {b: g.sites(b) for b in set(cheap) | set(spread)}
    norms = g.canonize_compress_norm(maxdim)
    assert norms.shape == (512,) and np.all(np.isfinite(norms)) and np.all(norms > 0)
    worst = 0.0
    for b in cheap:
        p = O.OMPS([a.copy() for a in init[b]])
        O.canonize(p, O.MixedCanonical(Ls[b]))
        O.compress(p, maxdim=maxdim[b])
        worst = max(worst, abs(norms[b] - O.norm(p)) / O.norm(p))
    worst_dev, devs = 0.0, []
    for b in spread:
        psi = tenetgb.MPS([a.copy() for a in init[b]], ctx=ctx)
        psi.canonize_(tenetgb.MixedCanonical(Ls[b]))
        psi.compress_(maxdim=maxdim[b])
        devs.append((int(chis[b]), abs(norms[b] - psi.norm()) / psi.norm()))
        worst_dev = max(worst_dev, devs[-1][1])
        del psi
    print(f"\n512-MPS population: norms vs oracle (150 cheapest) {worst:.2e}; vs per-instance device path "
          f"(12, χ {min(chis[b] for b in spread)}..{max(chis[b] for b in spread)}) {worst_dev:.2e}; "
          + ", ".join(f"χ={c}: {e:.1e}" for c, e in devs))
    assert worst <= 1e-12 and worst_dev <= 1e-10
