"""Algorithmic work conventions for every figure the bench reports: the counts depend on
the shapes visited, never on the algorithm that runs (a Jacobi SVD is charged the
Golub–Reinsch count, a split-precision GEMM the complex product it stands for).

* complex multiply-add = 8 real flops; a complex GEMM m×n×k = 8·m·n·k;
* thin QR of a complex m×n (m ≥ n) = 4·(2mn² − ⅔n³) (LAWN 41, ×4 for complex), and the
  same again for forming Q;
* SVD of a complex m×n with U and V = 4·(4m²n + 8mn² + 9n³) (Golub–Van Loan's
  Golub–Reinsch count ×4; m ≥ n after transposing);
* a permutation moves 2·numel·itemsize bytes;
* a split-BF16 (Ozaki) GEMM issues S(S+1)/2 plane pairs of real tensor-core products
  2·(2m)·n·(2k) each (the kernel-level rate), while end-to-end throughput counts only the
  complex product 8·m·n·k.

The TEBD gate follows the reference's sequence (`simple_update.jl:20-77` with the centre
moved by `canonize!`, two QR gauge moves per gate): θ = A·B, the gate on the physical
pair, the SVD of θ (χ_l d × d χ_r), and two QRs of (χ d × χ) sites with their R·B
products.
"""

from __future__ import annotations


def gemm(m, n, k):
    return 8.0 * m * n * k


def qr(m, n, form_q=True):
    if m < n:
        m, n = n, m
    f = 4.0 * (2.0 * m * n * n - 2.0 * n**3 / 3.0)
    return 2.0 * f if form_q else f


def svd(m, n):
    if m < n:
        m, n = n, m
    return 4.0 * (4.0 * m * m * n + 8.0 * m * n * n + 9.0 * n**3)


def permute_bytes(numel, itemsize):
    return 2.0 * numel * itemsize


def split_gemm_tensor_flops(m, n, k, planes=8):
    """Real tensor-core flops a split-BF16 complex GEMM issues (plane pairs p + q < S)."""
    return planes * (planes + 1) / 2.0 * 2.0 * (2 * m) * n * (2 * k)


def tebd_gate(chl, chm, chr, d=2):
    """One two-site gate on bonds (χ_l, χ_m, χ_r): two QR gauge moves of (χ d × χ) sites
    with their R·B products, θ = A·B, the gate, the SVD of θ."""
    m, n = chl * d, d * chr
    moves = 2.0 * (qr(chl * d, chm) + gemm(chm, d * chr, chm))
    return moves + gemm(m, n, chm) + gemm(chl * chr, d * d, d * d) + svd(m, n)


def tebd_layer(bonds, start, n_gates, d=2):
    """A brickwork layer on an MPS with bond dimensions ``bonds`` (length L−1, bond i
    between sites i and i+1, 1-based sites), gates on sites (start + 2g, start + 2g + 1).
    Brickwork gates leave each other's outer bonds alone, so the pre-layer bonds give
    every gate's θ shape."""
    b = [1] + list(bonds) + [1]
    tot = 0.0
    for g in range(n_gates):
        a = start + 2 * g
        tot += tebd_gate(b[a - 1], b[a], b[a + 1], d)
    return tot


def canonize_compress(L, bonds, maxdim, d=2):
    """canonize!(ψ, site L) → compress!(ψ; maxdim) → norm on one MPS (config 4): a QR
    sweep left→right, an LQ sweep right→left, an SVD sweep left→right with truncation."""
    b = [1] + list(bonds) + [1]
    tot = 0.0
    for k in range(1, L):
        tot += qr(b[k - 1] * d, b[k]) + gemm(b[k], d * b[k + 1], b[k])
    for i in range(L, 1, -1):
        tot += qr(d * b[i], b[i - 1]) + gemm(b[i - 2] * d, b[i - 1], b[i - 1])
    prev = 1
    for k in range(1, L):
        m, n = prev * d, b[k]
        r = min(maxdim, m, n)
        tot += svd(m, n) + gemm(r, n, m) + gemm(r, d * b[k + 1], n)
        prev = r
    return tot
