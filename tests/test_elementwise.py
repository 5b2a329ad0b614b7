"""Banded elementwise algebra on the GPU: axpy!(a, X, Y), A + B, A - B, alpha * A,
A + sigma I and dot(x, A, y), against the reference's rules and OpenBLAS.

* Equal bandwidths: axpy!(a, X.data, Y.data) -- BLAS daxpy over the storage, which
  OpenBLAS fuses -- so the result equals daxpy's (the golden file) bit for bit.
* Different bandwidths: banded_generic_axpy! -- BandError (Y untouched) when X has a
  nonzero outside Y's bands, else a*x + y rounded twice on the overlapping bands: bit for
  bit with NumPy's unfused evaluation.
* dot(x, A, y): a deterministic tree sum, equal to the dense x' A y to 1e-13 relative.
Cases follow test/test_broadcasting.jl (axpy between different bandwidths, BandError)
and test/test_dot.jl.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
NEXT = os.path.join(os.path.dirname(__file__), "golden", "next_golden.npz")


def _dev(bm, gpu, data, m, l, u):
    A = bm.BandedMatrix(bm.band_storage(l + u + 1, data.shape[1], torch.float64, gpu), m, l, u)
    A.data.copy_(torch.from_numpy(np.ascontiguousarray(data)))
    return A


def test_axpy_and_dot_golden(bm, gpu):
    gn = np.load(NEXT)
    for c in range(2):
        m, n, xl, xu, yl, yu = (int(v) for v in gn[f"ax{c}_dims"])
        a = float(gn[f"ax{c}_a"][0])
        X = _dev(bm, gpu, gn[f"ax{c}_X"], m, xl, xu)
        Y = _dev(bm, gpu, gn[f"ax{c}_Y"], m, yl, yu)
        bm.axpy_(a, X, Y)
        assert np.array_equal(Y.data.cpu().numpy(), gn[f"ax{c}_Z"]), c
        d = float(bm.dot(torch.from_numpy(gn[f"ax{c}_x"]).to(gpu), X, torch.from_numpy(gn[f"ax{c}_y"]).to(gpu)))
        ref = float(gn[f"ax{c}_dot"][0])
        assert abs(d - ref) <= 1e-13 * max(1.0, abs(ref))


def test_axpy_band_error_leaves_y_untouched(bm, gpu):
    rng = np.random.default_rng(1)
    m = n = 50
    X = _dev(bm, gpu, rng.standard_normal((1 + 3 + 1, n)), m, 1, 3)  # (1, 3): band 3 is nonzero
    Y = _dev(bm, gpu, rng.standard_normal((2 + 1 + 1, n)), m, 2, 1)  # (2, 1)
    before = Y.data.clone()
    with pytest.raises(bm.BandError):
        bm.axpy_(2.0, X, Y)
    assert torch.equal(Y.data, before)
    # zero the extra bands of X: the same call succeeds on the overlap
    X.data[0:2, :] = 0.0
    bm.axpy_(2.0, X, Y)
    Xd, Yd = X.to_dense().cpu().numpy(), bm.BandedMatrix(before, m, 2, 1).to_dense().cpu().numpy()
    assert np.array_equal(Y.to_dense().cpu().numpy(), 2.0 * Xd + Yd)


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_add_sub_scale_shift_dot(bm, gpu, dt):
    rng = np.random.default_rng(2)
    m, n = 300, 280
    A = bm.brandn(dt, m, n, 3, 2, device=gpu)
    B = bm.brandn(dt, m, n, 1, 5, device=gpu)
    Ad, Bd = A.to_dense(), B.to_dense()
    for R, ref in ((A + B, Ad + Bd), (A - B, Ad - Bd), (2.5 * A, 2.5 * Ad), (-B, -Bd)):
        assert torch.equal(R.to_dense(), ref)
    assert (A + B).bandwidths() == (3, 5)
    S = A.copy()
    bm.shift_(S, 7.0)
    assert torch.equal(S.to_dense(), Ad + 7.0 * torch.eye(m, n, dtype=dt, device=gpu))
    x = torch.from_numpy(rng.standard_normal(m)).to(gpu, dt)
    y = torch.from_numpy(rng.standard_normal(n)).to(gpu, dt)
    y[5] = 0.0
    d = float(bm.dot(x, A, y))
    ref = float((x.double() @ (Ad.double() @ y.double())))
    tol = 1e-13 if dt == torch.float64 else 1e-5
    assert abs(d - ref) <= tol * float((x.double().abs() @ (Ad.double().abs() @ y.double().abs())))
