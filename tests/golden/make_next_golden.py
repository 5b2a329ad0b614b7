"""Generate tests/golden/next_golden.npz: OpenBLAS results for the routines beside the
main path (triangular band solve and product, banded x dense and dense x banded
products, symmetric band product, banded Cholesky), from SciPy's bundled OpenBLAS --
the library family BandedMatrices.jl ccalls for them:
  * tbmv / tbsv, every uplo / trans / diag form   (tbmv!/tbsv!, src/blas.jl:71-147)
  * banded x dense: one dgbmv 'N' per column       (src/generic/matmul.jl:243-256)
  * dense x banded: one dgbmv 'T' per row          (src/generic/matmul.jl:258-271)
  * sbmv, upper / lower                            (sbmv!, src/blas.jl:35-64)
  * pbtrf / pbtrs, upper / lower                   (pbtrf!/pbtrs!, src/lapack.jl:268-332,
                                                    banded_chol!, src/symbanded/BandedCholesky.jl:2-12)
Inputs are NumPy PCG64 streams, stored beside the outputs.

Run:  python tests/golden/make_next_golden.py
"""
from __future__ import annotations

import os

import numpy as np
from scipy.linalg import blas, lapack

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "next_golden.npz")
FORMS = [(u, t, d) for u in "UL" for t in "NT" for d in "NU"]


def main():
    g = {}
    rng = np.random.default_rng(8080)
    for c, (n, k) in enumerate([(200, 7), (150, 40)]):
        for u, t, d in FORMS:
            key = f"tri{c}_{u}{t}{d}"
            A = rng.standard_normal((k + 1, n))
            A[k if u == "U" else 0] += 4.0 * np.sign(A[k if u == "U" else 0])  # a stable solve
            x = rng.standard_normal(n)
            kw = dict(lower=int(u == "L"), trans=int(t == "T"), diag=int(d == "U"))
            g[key + "_A"], g[key + "_x"] = A, x
            g[key + "_mv"] = blas.dtbmv(k, np.asfortranarray(A), x.copy(), **kw)
            g[key + "_sv"] = blas.dtbsv(k, np.asfortranarray(A), x.copy(), **kw)
        g[f"tri{c}_dims"] = np.array([n, k], dtype=np.int64)
    # banded x dense and dense x banded (the reference's per-column / per-row dgbmv)
    for c, (m, n, kl, ku, k) in enumerate([(120, 100, 3, 5, 7), (64, 80, 20, 2, 3)]):
        A = rng.standard_normal((kl + ku + 1, n))
        B = rng.standard_normal((n, k))
        C0 = rng.standard_normal((m, k))
        D = rng.standard_normal((k, m))
        E0 = rng.standard_normal((k, n))
        alpha, beta = 0.75, -0.5
        C = np.stack([blas.dgbmv(m, n, kl, ku, alpha, np.asfortranarray(A), B[:, j], beta=beta, y=C0[:, j].copy())
                      for j in range(k)], axis=1)
        E = np.stack([blas.dgbmv(m, n, kl, ku, alpha, np.asfortranarray(A), D[r, :], beta=beta, y=E0[r, :].copy(),
                                 trans=1) for r in range(k)], axis=0)
        g[f"bd{c}_dims"] = np.array([m, n, kl, ku, k], dtype=np.int64)
        g[f"bd{c}_ab"] = np.array([alpha, beta])
        g[f"bd{c}_A"], g[f"bd{c}_B"], g[f"bd{c}_C0"], g[f"bd{c}_C"] = A, B, C0, C
        g[f"bd{c}_D"], g[f"bd{c}_E0"], g[f"bd{c}_E"] = D, E0, E
    # symmetric band product and banded Cholesky (a diagonally dominant SPD band)
    for c, (n, k) in enumerate([(300, 6), (200, 40)]):
        for u in "UL":
            key = f"sym{c}_{u}"
            A = rng.standard_normal((k + 1, n))
            A[k if u == "U" else 0] = np.abs(A[k if u == "U" else 0]) + 2.0 * (k + 1)
            x, y0 = rng.standard_normal(n), rng.standard_normal(n)
            b = rng.standard_normal((n, 2))
            g[key + "_A"], g[key + "_x"], g[key + "_y0"], g[key + "_b"] = A, x, y0, b
            g[key + "_sbmv"] = blas.dsbmv(k, 0.7, np.asfortranarray(A), x, beta=-1.5, y=y0.copy(), lower=int(u == "L"))
            F, info = lapack.dpbtrf(np.asfortranarray(A), lower=int(u == "L"))
            assert info == 0
            X, info = lapack.dpbtrs(F, b, lower=int(u == "L"))
            g[key + "_F"], g[key + "_X"] = F, X
        g[f"sym{c}_dims"] = np.array([n, k], dtype=np.int64)
    # axpy!: equal bandwidths is BLAS daxpy over the storage; different bandwidths is
    # banded_generic_axpy!'s a*x + y on the overlapping bands (NumPy does not fuse); dot
    for c, (m, n, xl, xu, yl, yu) in enumerate([(90, 90, 3, 4, 3, 4), (80, 100, 2, 5, 6, 1)]):
        X = rng.standard_normal((xl + xu + 1, n))
        Y = rng.standard_normal((yl + yu + 1, n))
        a = -0.625
        if (xl, xu) == (yl, yu):
            Z = blas.daxpy(X.ravel(order="F"), Y.ravel(order="F").copy(), a=a).reshape(Y.shape, order="F")
        else:
            Z = Y.copy()
            for j in range(n):
                for k in range(max(0, j - min(xu, yu)), min(m, j + min(xl, yl) + 1)):
                    Z[yu + k - j, j] = a * X[xu + k - j, j] + Y[yu + k - j, j]
            for j in range(n):  # the test keeps X's extra bands zero, as banded_generic_axpy! requires
                for k in range(max(0, j - xu), min(m, j + xl + 1)):
                    if not (-yu <= k - j <= yl):
                        X[xu + k - j, j] = 0.0
        x, y = rng.standard_normal(m), rng.standard_normal(n)
        Xd = np.zeros((m, n))
        for j in range(n):
            for k in range(max(0, j - xu), min(m, j + xl + 1)):
                Xd[k, j] = X[xu + k - j, j]
        g[f"ax{c}_dims"] = np.array([m, n, xl, xu, yl, yu], dtype=np.int64)
        g[f"ax{c}_a"] = np.array([a])
        g[f"ax{c}_X"], g[f"ax{c}_Y"], g[f"ax{c}_Z"] = X, Y, Z
        g[f"ax{c}_x"], g[f"ax{c}_y"], g[f"ax{c}_dot"] = x, y, np.array([x @ (Xd @ y)])
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB, {len(g)} arrays)")


if __name__ == "__main__":
    main()
