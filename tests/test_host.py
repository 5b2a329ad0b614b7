"""Host-side logic of the Python mirror, on CPU tensors: band storage layout and the
BandedMatrix constructors (src/banded/BandedMatrix.jl:16-68, 222-232), the PDE operator
assembly, and the batched solver's longest-first schedules.  No GPU and no library call."""
import numpy as np
import pytest
import torch


def _dense_band(rng, m, n, l, u):
    A = np.zeros((m, n))
    for j in range(n):
        for i in range(max(0, j - u), min(m, j + l + 1)):
            A[i, j] = rng.standard_normal()
    return A


@pytest.mark.parametrize("m,n,l,u", [(7, 7, 2, 1), (9, 5, 3, 0), (5, 9, 0, 4), (6, 6, 0, 0), (4, 10, 1, 6)])
def test_band_storage_round_trip(bm, m, n, l, u):
    rng = np.random.default_rng(m * 100 + n * 10 + l + u)
    A = torch.from_numpy(_dense_band(rng, m, n, l, u))
    B = bm.BandedMatrix.from_dense(A, (l, u))
    assert B.shape == (m, n) and bm.bandwidths(B) == (l, u)
    assert B.data.shape == (l + u + 1, n) and B.data.stride(0) == 1 and B.lda >= l + u + 1
    # A[k, j] = data[u + k - j, j] (src/banded/BandedMatrix.jl:414-419)
    for j in range(n):
        for k in range(max(0, j - u), min(m, j + l + 1)):
            assert B.data[u + k - j, j].item() == A[k, j].item()
    assert torch.equal(B.to_dense(), A)
    W = B.rewiden((l + 2, u + 1))
    assert bm.bandwidths(W) == (l + 2, u + 1) and torch.equal(W.to_dense(), A)
    with pytest.raises(Exception):
        B.rewiden((max(l - 1, 0) if l else -1, u))


def test_band_storage_with_padding(bm):
    d = bm.band_storage(3, 6, torch.float64, "cpu", lda=5, fill=0.0)
    assert d.shape == (3, 6) and d.stride() == (1, 5)
    B = bm.BandedMatrix(d, 6, 1, 1)
    assert B.lda == 5


def test_diffusion_operator_assembly(bm):
    """The 5-point variable-coefficient operator in natural ordering (harmonic face means,
    boundary faces taking the cell value) against a cell-by-cell dense assembly."""
    G = 5
    kc = np.exp(bm.pde.gaussian_field(G, 2.0, seed=3))
    A = bm.pde.diffusion_band(kc, torch.float64, "cpu")
    assert A.shape == (G * G, G * G) and bm.bandwidths(A) == (G, G)
    D = np.zeros((G * G, G * G))
    hm = lambda a, b: 2 * a * b / (a + b)
    for i in range(G):
        for j in range(G):
            p = i * G + j
            for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                ii, jj = i + di, j + dj
                if 0 <= ii < G and 0 <= jj < G:
                    f = hm(kc[i, j], kc[ii, jj])
                    D[p, ii * G + jj] = -f
                    D[p, p] += f
                else:
                    D[p, p] += kc[i, j]
    Ad = A.to_dense().numpy()
    assert np.allclose(Ad, D, rtol=1e-14, atol=0)
    assert np.array_equal(Ad, Ad.T)
    # weakly diagonally dominant; strictly on the boundary cells (their outer faces)
    off = np.abs(Ad).sum(1) - np.diag(Ad)
    assert (np.diag(Ad) >= off * (1 - 1e-14)).all()
    edge = np.zeros((G, G), bool)
    edge[0, :] = edge[-1, :] = edge[:, 0] = edge[:, -1] = True
    assert (np.diag(Ad)[edge.ravel()] > off[edge.ravel()]).all()


def test_gaussian_field_is_seeded_and_normalised(bm):
    g1 = bm.pde.gaussian_field(64, 16.0, seed=11)
    g2 = bm.pde.gaussian_field(64, 16.0, seed=11)
    assert np.array_equal(g1, g2)
    assert abs(g1.mean()) < 1e-12 and abs(g1.std() - 1.0) < 1e-12
    # correlation length 16 cells: neighbours are strongly correlated
    assert np.corrcoef(g1[:, :-1].ravel(), g1[:, 1:].ravel())[0, 1] > 0.9


def test_longest_first_orders(bm):
    from importlib import import_module

    batched = import_module(bm.__name__ + ".batched")
    rng = np.random.default_rng(5)
    n = rng.integers(10, 2000, 300)
    kl = rng.integers(0, 40, 300)
    ku = rng.integers(0, 40, 300)
    nrhs = rng.integers(1, 9, 300)
    cost = n * (2 * kl * (kl + ku) + kl) + nrhs * 2 * n * (2 * kl + ku + 1)
    order = batched.lpt_order(n, kl, ku, nrhs)
    assert sorted(order.tolist()) == list(range(300))
    assert (np.diff(cost[order]) <= 0).all()
    order2, n_wide = batched.schedule_order(n, kl, ku, nrhs, narrow_cols=24)
    assert sorted(order2.tolist()) == list(range(300))
    wide = (kl + ku + 1) > 24
    assert n_wide == int(wide.sum())
    assert wide[order2[:n_wide]].all() and not wide[order2[n_wide:]].any()
    assert (np.diff(cost[order2[:n_wide]]) <= 0).all() and (np.diff(cost[order2[n_wide:]]) <= 0).all()


def test_scalar_indexing_semantics(bm):
    """A[k, j] reads the band entry or zero outside the band; A[k, j] = v writes in-band
    entries, accepts zero outside the band and raises BandError otherwise
    (src/banded/BandedMatrix.jl:414-442, 627-643); out-of-range indices raise IndexError."""
    rng = np.random.default_rng(9)
    m, n, l, u = 7, 6, 2, 1
    Ad = _dense_band(rng, m, n, l, u)
    A = bm.BandedMatrix.from_dense(torch.from_numpy(Ad), (l, u))
    for k in range(m):
        for j in range(n):
            assert A[k, j] == Ad[k, j]
    A[3, 2] = 5.0  # in band (j - k = -1)
    assert A[3, 2] == 5.0 and A.data[u + 3 - 2, 2].item() == 5.0
    A[0, 5] = 0.0  # outside the band, zero: accepted, nothing stored
    with pytest.raises(bm.BandError):
        A[0, 5] = 1.0
    with pytest.raises(bm.BandError):
        A[6, 0] = -2.0
    with pytest.raises(IndexError):
        A[7, 0]
    with pytest.raises(IndexError):
        A[0, -1] = 0.0


def test_random_constructors_and_bandwidth(bm):
    """brand fills every storage slot, the off-matrix corners included, from [0, 1); brandn
    from the standard normal (src/banded/BandedMatrix.jl:184-204); bandwidth(A, 1) = l,
    bandwidth(A, 2) = u."""
    g = torch.Generator().manual_seed(4)
    A = bm.brand(torch.float64, 300, 200, 3, 5, device="cpu", generator=g)
    assert A.shape == (300, 200) and bm.bandwidths(A) == (3, 5)
    assert bm.bandwidth(A, 1) == 3 and bm.bandwidth(A, 2) == 5
    d = bm.bandeddata(A)
    assert d.shape == (9, 200) and bool((d >= 0).all()) and bool((d < 1).all())
    assert abs(d.mean().item() - 0.5) < 0.02
    B = bm.brandn(torch.float32, 200, 200, 2, 2, device="cpu", generator=g)
    assert B.dtype == torch.float32 and abs(B.data.mean().item()) < 0.05 and abs(B.data.std().item() - 1) < 0.05
    Z = bm.BandedMatrix.zeros((5, 4), (1, 2), torch.float64, "cpu")
    assert torch.equal(Z.to_dense(), torch.zeros(5, 4, dtype=torch.float64))


@pytest.mark.parametrize("n,l,u", [(40, 3, 2), (25, 0, 4), (30, 5, 0), (12, 11, 11)])
def test_banded_lu_views(bm, orc, n, l, u):
    """BandedLU's p, L and U views (src/banded/BandedLU.jl:114-130) rebuilt from gbtrf
    factors and pivots (here the oracle's xGBTF2 on a non-dominant band, so rows are
    interchanged): A[p, :] == L U, L unit lower triangular, U upper triangular with
    bandwidth l + u."""
    from importlib import import_module

    lu_mod = import_module(bm.__name__ + ".lu")
    rng = np.random.default_rng(n * 7 + l + u)
    data = rng.standard_normal((l + u + 1, n))
    LU, ipiv, info = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    assert info == 0 and (ipiv != np.arange(1, n + 1)).any() or l == 0
    F = lu_mod.BandedLU(bm.BandedMatrix(torch.from_numpy(np.ascontiguousarray(LU.T)).t(), n, l, l + u),
                        torch.from_numpy(ipiv), torch.tensor([info]), l, u)
    A = orc.band_to_dense(data, n, l, u)
    Lm, Um, p = F.L, F.U, F.p
    assert sorted(p.tolist()) == list(range(1, n + 1))
    assert np.allclose(A[p - 1, :], Lm @ Um, rtol=1e-12, atol=1e-12)
    assert np.array_equal(np.diag(Lm), np.ones(n)) and np.array_equal(Lm, np.tril(Lm))
    assert np.array_equal(Um, np.triu(Um)) and np.array_equal(Um, np.tril(Um, l + u))
    assert F.issuccess() and F.size() == (n, n)


def test_product_bandwidths(bm):
    """prodbandwidths (src/generic/utils.jl:19-21): sums of the factors' bandwidths, (0, 0)
    for no factor, a single factor's own bandwidths; negative bandwidths add too."""
    from importlib import import_module

    gbmm = import_module(bm.__name__ + ".gbmm")
    A = bm.BandedMatrix.zeros((6, 6), (2, 1), torch.float64, "cpu")
    B = bm.BandedMatrix.zeros((6, 6), (0, 3), torch.float64, "cpu")
    C = bm.BandedMatrix(torch.zeros(0, 6, dtype=torch.float64), 6, -1, -1)
    assert gbmm.prodbandwidths() == (0, 0)
    assert gbmm.prodbandwidths(A) == (2, 1)
    assert gbmm.prodbandwidths(A, B) == (2, 4)
    assert gbmm.prodbandwidths(A, B, A) == (4, 5)
    assert gbmm.prodbandwidths(A, C) == (1, 0)
