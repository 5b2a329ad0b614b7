"""Adjoint of x = A \\ b (bm_{d,s}gbsv_adjoint via banded_solve): against central finite
differences (h = 1e-6), the FP64 reference gradient of the oracle, and torch's gradcheck;
on random bands and on the 5-point variable-coefficient diffusion operator."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_adjoint_vs_oracle_and_fd_random(bm, gpu, orc):
    rng = np.random.default_rng(1)
    n, l, u = 300, 5, 3
    data = rng.standard_normal((l + u + 1, n))
    data[u] += 6.0
    b = rng.standard_normal(n)
    w = rng.standard_normal(n)
    D = torch.from_numpy(data).to(gpu).requires_grad_(True)
    bt = torch.from_numpy(b).to(gpu).requires_grad_(True)
    x = bm.banded_solve(D, bt, l, u)
    (x * torch.from_numpy(w).to(gpu)).sum().backward()
    gb, gD = bt.grad.cpu().numpy(), D.grad.cpu().numpy()
    LU, ipiv, _ = orc.gbtf2(n, n, l, u, orc.lu_storage(data, n, l, u))
    xr = orc.gbtrs("N", n, l, u, LU, ipiv, b)
    gbr, gDr = orc.gb_adjoint(n, l, u, LU, ipiv, xr, w)
    assert np.abs(gb - gbr).max() <= 1e-12 * np.abs(gbr).max()
    assert np.abs(gD - gDr).max() <= 1e-12 * np.abs(gDr).max()

    def loss(dat, bb):
        LU, ip, _ = orc.gbtf2(n, n, l, u, orc.lu_storage(dat, n, l, u))
        return float(w @ orc.gbtrs("N", n, l, u, LU, ip, bb))

    h = 1e-6
    for i in (0, 17, n - 1):
        e = np.zeros(n)
        e[i] = h
        fd = (loss(data, b + e) - loss(data, b - e)) / (2 * h)
        assert abs(fd - gb[i]) <= 1e-6 * max(1.0, abs(fd))
    for (r, j) in ((u, 10), (0, 50), (l + u, 7), (u + 2, 200)):
        dp, dm = data.copy(), data.copy()
        dp[r, j] += h
        dm[r, j] -= h
        fd = (loss(dp, b) - loss(dm, b)) / (2 * h)
        assert abs(fd - gD[r, j]) <= 1e-6 * max(1.0, abs(fd)), (r, j)


def test_adjoint_recompute_x_and_multi_rhs(bm, gpu):
    rng = np.random.default_rng(2)
    n, l, u = 200, 4, 6
    data = rng.standard_normal((l + u + 1, n))
    data[u] += 8.0
    B = rng.standard_normal((n, 3))
    W = rng.standard_normal((n, 3))
    grads = []
    for rec in (False, True):
        D = torch.from_numpy(data).to(gpu).requires_grad_(True)
        Bt = torch.from_numpy(B).to(gpu).requires_grad_(True)
        X = bm.banded_solve(D, Bt, l, u, recompute_x=rec)
        (X * torch.from_numpy(W).to(gpu)).sum().backward()
        grads.append((D.grad.clone(), Bt.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0]) and torch.equal(grads[0][1], grads[1][1])


def test_adjoint_gradcheck(bm, gpu):
    rng = np.random.default_rng(3)
    n, l, u = 9, 2, 1
    data = rng.standard_normal((l + u + 1, n))
    data[u] += 4.0
    D = torch.from_numpy(data).to(gpu).requires_grad_(True)
    b = torch.from_numpy(rng.standard_normal(n)).to(gpu).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda d, bb: bm.banded_solve(d, bb, l, u), (D, b), eps=1e-6, atol=1e-7)


@pytest.mark.parametrize("G", [16, 48])
def test_adjoint_pde(bm, gpu, orc, G):
    """5-point diffusion, coefficient exp(g) with g a Gaussian field of correlation length
    16 cells: directional finite differences (h = 1e-6) of L = w.x and the FP64 reference."""
    kcell = np.exp(bm.pde.gaussian_field(G, 16.0, seed=G))
    A = bm.pde.diffusion_band(kcell, torch.float64, gpu)
    n = G * G
    rng = np.random.default_rng(G)
    b = torch.from_numpy(rng.standard_normal(n)).to(gpu)
    w = torch.from_numpy(rng.standard_normal(n)).to(gpu)
    D = A.data.clone().requires_grad_(True)
    bt = b.clone().requires_grad_(True)
    x = bm.banded_solve(D, bt, G, G)
    (x * w).sum().backward()
    data = A.data.cpu().numpy()
    LU, ipiv, _ = orc.gbtf2(n, n, G, G, orc.lu_storage(data, n, G, G))
    xr = orc.gbtrs("N", n, G, G, LU, ipiv, b.cpu().numpy())
    gbr, gDr = orc.gb_adjoint(n, G, G, LU, ipiv, xr, w.cpu().numpy())
    assert np.abs(bt.grad.cpu().numpy() - gbr).max() <= 1e-10 * np.abs(gbr).max()
    assert np.abs(D.grad.cpu().numpy() - gDr).max() <= 1e-10 * np.abs(gDr).max()
    # directional derivative along a random band direction and a random b direction
    h = 1e-6
    dD = torch.from_numpy(rng.standard_normal(data.shape)).to(gpu) * (A.data != 0)
    db = torch.from_numpy(rng.standard_normal(n)).to(gpu)

    def L(d, bb):
        return float((bm.banded_solve(d, bb, G, G) * w).sum())

    fd = (L(A.data + h * dD, b + h * db) - L(A.data - h * dD, b - h * db)) / (2 * h)
    ad = float((D.grad * dD).sum() + (bt.grad * db).sum())
    assert abs(fd - ad) <= 1e-6 * max(1.0, abs(fd)), (fd, ad)
