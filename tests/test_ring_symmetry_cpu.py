"""The symmetries the ring kernel (dst.cu k_ring_edge) relies on, checked on the CPU with the
tables built as the library builds them.

* W[j][k] = 2 sin(pi (j+1)(k+1)/M) (the DST-I matrix, dst_matrix_table): row N-1-j equals
  (-1)^k times row j, so a mode row's inverse transform at a point and at its mirror image is
  e + o and e - o (e, o: the sums over even and odd modes).
* E = W P (dst_edge_matrix; P puts the coarse row get_bc reads, operators_fluid.F90:475-535, on
  a finer level's edge entries): E[k][k'] vanishes unless k and k' have the same parity, so only
  those entries are kept.
"""
import numpy as np
import pytest

PI = np.longdouble("3.141592653589793238462643383279502884")


def _w(m):
    M, N = m, m - 1
    r = np.arange(2 * M, dtype=np.longdouble)
    tab = (2 * np.sin(PI * r / np.longdouble(M))).astype(np.float64)
    j = np.arange(1, N + 1)
    return tab[np.outer(j, j) % (2 * M)]


def _edge(m, W):
    N, mq = m - 1, m // 4
    P = np.zeros((N, N))
    for jj in range(N):
        p = jj + 1
        r0 = mq - 1 + p // 2
        P[jj] = 0.5 * (W[r0] + W[r0 + 1]) if p & 1 else W[r0]
    return W @ P


@pytest.mark.parametrize("m", [32, 64, 96, 256])
def test_dst_rows_mirror(m):
    W = _w(m)
    N = m - 1
    sign = (-1.0) ** np.arange(N)
    assert np.abs(W[::-1, :] - W * sign[None, :]).max() <= 4 * np.finfo(float).eps
    # the pair from one pass: e + o and e - o against the two direct dot products
    rng = np.random.default_rng(m)
    s = rng.standard_normal(N)
    for r in (m // 4 - 1, m // 4 + 3, m // 2 - 1):
        e, o = W[r, 0::2] @ s[0::2], W[r, 1::2] @ s[1::2]
        assert abs((e + o) - W[r] @ s) <= 1e-13 * np.abs(W[r] * s).sum()
        assert abs((e - o) - W[N - 1 - r] @ s) <= 1e-13 * np.abs(W[r] * s).sum()


@pytest.mark.parametrize("m", [32, 64, 96, 256])
def test_edge_matrix_parity(m):
    W = _w(m)
    E = _edge(m, W)
    N = m - 1
    cross = (np.arange(N)[:, None] + np.arange(N)[None, :]) % 2 == 1
    # zero up to the round-off of the product (N terms of size up to 4)
    assert np.abs(E[cross]).max() <= 8 * N * np.finfo(float).eps * np.abs(E).max()
    assert np.abs(E[~cross]).max() > 1.0
