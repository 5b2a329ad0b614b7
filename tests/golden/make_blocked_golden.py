"""Generate tests/golden/blocked_golden.npz: OpenBLAS dgbtrf/dgbtrs results in the
blocked regime, at the bandwidths of the wide-band workloads.

OpenBLAS (SciPy's bundled build, the library family BandedMatrices.jl ccalls through
LAPACK.gbtrf!/gbtrs!, src/banded/BandedLU.jl:98 and src/banded/linalg.jl:28) switches
from unblocked dgbtf2 to blocked dgbtrf once kl reaches its block size: the trailing
updates then run as dgemm/dtrsm, in a different order from the column-by-column
factorization.  These vectors pin the GPU's pivots (bit for bit) and factors (to a
stated tolerance) in that regime:
  * c4a  -- n = 8192, l = u = 128, entries randn-like, + 16 on the diagonal (the recipe
            of the n = 2^20, l = u = 128 refined-solve workload, at a smaller n);
  * c5   -- the 5-point variable-coefficient diffusion operator on a 512-wide, 8-high
            strip (n = 4096, l = u = 512, the bandwidth of the 512 x 512 PDE workload);
            the coefficient field exp(g), g a seeded Gaussian field of correlation
            length 16 cells, is stored in the file;
  * r512 -- n = 4096, l = u = 512, randn-like entries with no shift (pivoting on
            nearly every column).
"randn-like" entries are exactly reproducible on any machine: the sum of four PCG64
uniforms, centred and scaled to unit variance ((u1+u2)+(u3+u4)-2)*sqrt(3), with only
IEEE additions and multiplications (the tests regenerate them with the same function).
Stored per case: the OpenBLAS pivots (1-based, as offsets ipiv - 1 - j), the solution
of one right-hand side, and the factor storage of a few columns.

Run:  python tests/golden/make_blocked_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np
from scipy.linalg import lapack

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "blocked_golden.npz")


def randn_like(seed: int, shape) -> np.ndarray:
    """Unit-variance, exactly reproducible entries (see the module docstring)."""
    u = np.random.default_rng(seed).random((4,) + tuple(shape))
    return ((u[0] + u[1]) + (u[2] + u[3]) - 2.0) * np.sqrt(3.0)


def case_data(name: str, kfield=None):
    """(band data (l+u+1) x n, l, u, right-hand side) of a named case."""
    if name == "c4a":
        n, l = 8192, 128
        data = randn_like(41, (2 * l + 1, n))
        data[l] += 16.0
        return data, l, l, randn_like(42, (n,))
    if name == "r512":
        n, l = 4096, 512
        return randn_like(51, (2 * l + 1, n)), l, l, randn_like(52, (n,))
    if name == "c5":
        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        import __graft_entry__ as ge

        data = ge.package().pde.diffusion_band_data(kfield)
        G = kfield.shape[1]
        return data, G, G, randn_like(62, (data.shape[1],))
    raise KeyError(name)


def strip_field(G=512, H=8, corr=16.0, seed=61) -> np.ndarray:
    """exp(g) on an H x G strip: g is a G x G Gaussian field (correlation length corr
    cells, unit variance) restricted to its first H rows."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import __graft_entry__ as ge

    return np.exp(ge.package().pde.gaussian_field(G, corr, seed)[:H])


def main():
    g = {}
    kf = strip_field()
    g["c5_kfield"] = kf
    for name in ("c4a", "c5", "r512"):
        data, l, u, b = case_data(name, kf)
        n = data.shape[1]
        AB = np.zeros((2 * l + u + 1, n), order="F")
        AB[l:] = data
        LU, ipiv, info = lapack.dgbtrf(AB, l, u)
        assert info == 0
        x, info2 = lapack.dgbtrs(LU, l, u, b, ipiv)
        cols = np.linspace(0, n - 1, 16).astype(np.int64)
        g[f"{name}_dims"] = np.array([n, l, u], dtype=np.int64)
        g[f"{name}_pivoff"] = (ipiv - np.arange(n)).astype(np.uint16)  # ipiv (0-based) - j
        g[f"{name}_x"] = x
        g[f"{name}_cols"] = cols
        g[f"{name}_LUcols"] = np.asfortranarray(LU[:, cols])
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB, {len(g)} arrays)")


if __name__ == "__main__":
    main()
