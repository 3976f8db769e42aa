"""Index arithmetic of the linear-algebra kernels in ace-tn_gb300/csrc/linalg.cu,
restated in Python and checked exhaustively on the CPU (no kernel runs):

* jacobi_cluster_f32_kernel: the pairs of every local round are disjoint,
  every pair of rows is rotated exactly once per sweep, and the blocks are
  back at their home CTAs after the 2P-1 block rounds of a sweep;
* cholesky_kernel: the row-major enumeration of the upper-triangular 4x4
  tiles of the trailing matrix visits each tile once;
* slab_stage_kernel: the slabs partition the rows, the shared memory of one
  slab stays within the 227 KB a CTA can have for q <= 192, and the packed
  upper-triangle 4x4 Gram tiles, written by slab_reduce_kernel to a tile
  row and its mirror, cover every entry of G exactly once;
* double_layer_kernel (mixed.cu): division by multiplying with a
  host-computed reciprocal is exact below 2^16, and the shared-memory copy
  of A with its per-column offset tables gives the double-layer matrix.
"""

import itertools
import math

import pytest


def circle_pair(kk, r, n):
    """Pair kk of round r of the circle method on n (even) items, as in the
    kernels: position 0 fixed, the others rotating."""
    i0 = 0 if kk == 0 else ((kk - 1 + r) % (n - 1)) + 1
    k2 = n - 1 - kk
    j0 = 0 if k2 == 0 else ((k2 - 1 + r) % (n - 1)) + 1
    return i0, j0


def cluster_sweep(P, b):
    """One sweep of jacobi_cluster_f32_kernel: yields the pairs of each local
    round as global row pairs (block id * b + row), and the final layout."""
    lay = [[k, 2 * P - 1 - k] for k in range(P)]  # CTA k: (top, bottom) block ids
    rounds = []
    for t in range(2 * P - 1):
        nin = b - 1 if t == 0 else 0
        for lr in range(nin + b):
            pairs = []
            for k in range(P):
                top, bot = lay[k]
                for g in range(b):
                    if lr < nin:
                        half = 0 if g < b // 2 else 1
                        kk = g if half == 0 else g - b // 2
                        i0, j0 = circle_pair(kk, lr, b)
                        blk = top if half == 0 else bot
                        pairs.append((blk * b + i0, blk * b + j0))
                    else:
                        s = lr - nin
                        pairs.append((top * b + g, bot * b + (g + s) % b))
            rounds.append(pairs)
        nxt = [[None, None] for _ in range(P)]
        for k in range(P):
            top, bot = lay[k]
            if k == 0:
                nxt[0][0], nxt[1][0] = top, bot
            elif k < P - 1:
                nxt[k + 1][0], nxt[k - 1][1] = top, bot
            else:
                nxt[k][1], nxt[k - 1][1] = top, bot
        assert all(x is not None for row in nxt for x in row)
        lay = nxt
    return rounds, lay


@pytest.mark.parametrize("P,b", [(2, 4), (4, 4), (4, 20), (8, 12), (8, 4)])
def test_cluster_jacobi_visits_every_pair_once_per_sweep(P, b):
    rounds, lay = cluster_sweep(P, b)
    seen = {}
    for pairs in rounds:
        rows = [r for p in pairs for r in p]
        assert len(rows) == len(set(rows))  # disjoint pairs within a round
        for i, j in pairs:
            key = (min(i, j), max(i, j))
            assert i != j
            seen[key] = seen.get(key, 0) + 1
    n = 2 * P * b
    assert set(seen) == set(itertools.combinations(range(n), 2))
    assert all(v == 1 for v in seen.values())
    assert lay == [[k, 2 * P - 1 - k] for k in range(P)]
    # local rounds per sweep: b - 1 inside the blocks + (2P - 1) b across
    assert len(rounds) == (b - 1) + (2 * P - 1) * b


@pytest.mark.parametrize("q", [96, 100, 147, 160, 192, 224])
def test_cluster_jacobi_launch_shape(q):
    """Rows padded to a multiple of 8P (P = 8): b a multiple of 4, 8 b threads
    per CTA within the kernel's launch bound, four blocks of b rows of
    2 x ld floats within 227 KB where the cluster form is used."""
    P = 8
    qp = (q + 8 * P - 1) // (8 * P) * (8 * P)
    b = qp // (2 * P)
    ld = (q + 31) // 32 * 32
    assert b % 4 == 0 and 8 * b <= 256 and (8 * b) % 32 == 0
    smem = 4 * b * 2 * ld * 4
    assert ld > 256 or smem <= 227 * 1024


def tile_of(t, nbr):
    """cholesky_kernel's map from a linear index to an upper-triangular tile."""
    m = 2 * nbr + 1
    bi = int((m - math.sqrt(float(m * m - 8 * t))) * 0.5)
    bi = max(0, min(bi, nbr - 1))
    while bi + 1 < nbr and (bi + 1) * nbr - (bi + 1) * bi // 2 <= t:
        bi += 1
    while bi * nbr - bi * (bi - 1) // 2 > t:
        bi -= 1
    return bi, bi + (t - (bi * nbr - bi * (bi - 1) // 2))


@pytest.mark.parametrize("nbr", list(range(1, 50)) + [96, 128, 255])
def test_cholesky_upper_tiles_enumerated_once(nbr):
    tw = nbr * (nbr + 1) // 2
    tiles = [tile_of(t, nbr) for t in range(tw)]
    assert all(0 <= bi <= bk < nbr for bi, bk in tiles)
    assert len(set(tiles)) == tw


def slab_smem(q, rpb):
    """Dynamic shared memory of a slab stage: rpb rows of q rounded up to 4
    floats, and q rows of L^T padded to 32-float multiples."""
    ldq = (q + 3) // 4 * 4
    ldl = (q + 31) // 32 * 32
    return (rpb * ldq + q * ldl) * 4


def slab_rows(n, q, sms=152):
    rpb = (2 * n + sms - 1) // sms
    rpb = max(4, min(64, rpb))
    while rpb > 4 and slab_smem(q, rpb) > 227 * 1024:
        rpb -= 1
    return rpb


@pytest.mark.parametrize("n", [160, 1000, 3001, 5184, 12000, 65536])
@pytest.mark.parametrize("q", [32, 37, 147, 160, 192])
def test_slab_partition_and_shared_memory(n, q):
    if n < q:
        pytest.skip("n >= q")
    rpb = slab_rows(n, q)
    nblk = (n + rpb - 1) // rpb
    covered = sum(min(rpb, n - blk * rpb) for blk in range(nblk))
    assert covered == n and (nblk - 1) * rpb < n
    assert slab_smem(q, rpb) <= 227 * 1024
    if n == 5184 and q == 160:
        assert (rpb, nblk) == (64, 81)  # about two slabs per SM


def slab_tri_tile(t, nt4):
    """slab_tri_tile: tile t of the row-major upper triangle (diagonal
    included) of an nt4 x nt4 grid of 4 x 4 tiles (the float sqrt guess
    corrected by the loops)."""
    m = 2 * nt4 + 1
    bi = int((float(m) - math.sqrt(float(m * m - 8 * t))) * 0.5)
    bi = max(0, min(bi, nt4 - 1))
    while bi + 1 < nt4 and (bi + 1) * nt4 - (bi + 1) * bi // 2 <= t:
        bi += 1
    while bi * nt4 - bi * (bi - 1) // 2 > t:
        bi -= 1
    return bi, bi + (t - (bi * nt4 - bi * (bi - 1) // 2))


@pytest.mark.parametrize("q", [1, 5, 32, 37, 66, 147, 160, 192])
def test_packed_gram_tiles_cover_g_once(q):
    """Each float4 entry e of a packed partial is tile e // 4, tile row e % 4;
    the reduction writes the row's in-range entries and, off the diagonal
    tiles, their mirrors."""
    nt4 = (q + 3) // 4
    ne = nt4 * (nt4 + 1) // 2 * 4
    written = {}
    for e in range(ne):
        ti, tj = slab_tri_tile(e // 4, nt4)
        assert 0 <= ti <= tj < nt4
        row = 4 * ti + (e & 3)
        if row >= q:
            continue
        for cc in range(4):
            col = 4 * tj + cc
            if col < q:
                written[(row, col)] = written.get((row, col), 0) + 1
                if ti != tj:
                    written[(col, row)] = written.get((col, row), 0) + 1
    assert len(written) == q * q and set(written.values()) == {1}


@pytest.mark.parametrize("d", list(range(2, 66)) + [255, 4096, 65535])
def test_div16_reciprocal_is_exact(d):
    m = ((1 << 32) + d - 1) // d
    for x in list(range(0, 1 << 12)) + list(range((1 << 16) - 4096, 1 << 16)):
        assert (x * m) >> 32 == x // d


@pytest.mark.parametrize("D,d", [(2, 2), (3, 2), (4, 3), (6, 2)])
def test_double_layer_offset_tables(D, d):
    """The kernel's canonical copy of A (legs l, u, r, d, p, p fastest), the
    ket / bra offsets of column k = (l, L, u, U) and of row n = (r, R, dd, DD)
    give DL[n][k] = sum_p A[l,u,r,dd,p] A[L,U,R,DD,p]."""
    import numpy as np
    rng = np.random.default_rng(D * 10 + d)
    A = rng.standard_normal((D, D, D, D, d))
    D2, D4 = D * D, D ** 4
    c1 = D2 * d
    c0, c2, c3 = D * c1, D * d, d
    As = A.reshape(-1)  # [l][u][r][dd][p] is the canonical order
    k = np.arange(D4)
    U, u, L, l = k % D, (k // D) % D, (k // D2) % D, k // (D2 * D)
    kofs, bofs = l * c0 + u * c1, L * c0 + U * c1
    n = np.arange(D4)
    DD, dd, R, r = n % D, (n // D) % D, (n // D2) % D, n // (D2 * D)
    kn, bn = r * c2 + dd * c3, R * c2 + DD * c3
    dl = sum(As[kofs[None, :] + kn[:, None] + p] * As[bofs[None, :] + bn[:, None] + p]
             for p in range(d))
    ref = np.einsum("lurdp,LURDp->rRdDlLuU", A, A).reshape(D4, D4)
    assert np.abs(dl - ref).max() <= 1e-12 * np.abs(ref).max()
    assert (D4 * d + 2 * D4) * 4 <= 200 * 1024 or D > 10
