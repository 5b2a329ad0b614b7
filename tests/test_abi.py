"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(bm_\w+)\s*\(", src))
    return names


def test_header_declares_entry_points():
    names = _declared()
    assert "bm_dgbmv" in names and "bm_sgbmv" in names
    assert len(names) >= 4


def test_library_exports_every_declared_symbol(bm):
    lib = ctypes.CDLL(bm._lib.LIB_PATH)
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header(bm):
    declared = _declared()
    bound = set(bm._lib.SIGNATURES)
    assert declared == bound, f"header-only: {declared - bound}, binding-only: {bound - declared}"


def test_library_reports_version_without_gpu(bm):
    L = bm._lib.load()
    assert L.bm_version() >= 100
    assert isinstance(L.bm_last_error(), bytes)


def test_illegal_arguments_are_reported_before_any_device_call(bm):
    """LAPACK-style status (-i for the first illegal argument i), decided on the host, so
    it needs no GPU: the xGBMV / xGBTRF / xGBTRS checks the reference's LAPACK performs,
    and the refined batched solve's per-system pointer, tolerance and bandwidth checks."""
    L = bm._lib.load()
    P = ctypes.c_void_p
    fake = P(256)  # never dereferenced: every call below stops at an argument check
    s = P(0)
    # xgbmv(trans, m, n, kl, ku, alpha, A, lda, x, incx, beta, y, incy, stream)
    gbmv = lambda *a: L.bm_dgbmv(*a)
    assert gbmv(b"X", 4, 4, 1, 1, 1.0, fake, 3, fake, 1, 0.0, fake, 1, s) == -1
    assert gbmv(b"N", -1, 4, 1, 1, 1.0, fake, 3, fake, 1, 0.0, fake, 1, s) == -2
    assert gbmv(b"N", 4, -1, 1, 1, 1.0, fake, 3, fake, 1, 0.0, fake, 1, s) == -3
    assert gbmv(b"N", 4, 4, -1, 1, 1.0, fake, 3, fake, 1, 0.0, fake, 1, s) == -4
    assert gbmv(b"N", 4, 4, 1, 1, 1.0, fake, 2, fake, 1, 0.0, fake, 1, s) == -8
    assert gbmv(b"T", 4, 4, 1, 1, 1.0, fake, 3, fake, 0, 0.0, fake, 1, s) == -10
    assert gbmv(b"N", 4, 4, 1, 1, 1.0, fake, 3, fake, 1, 0.0, fake, 0, s) == -13
    # xgbtrf(m, n, kl, ku, AB, ldab, ipiv, info, stream)
    assert L.bm_dgbtrf(-1, 4, 1, 1, fake, 4, fake, fake, s) == -1
    assert L.bm_dgbtrf(4, -1, 1, 1, fake, 4, fake, fake, s) == -2
    assert L.bm_dgbtrf(4, 4, -1, 1, fake, 4, fake, fake, s) == -3
    assert L.bm_dgbtrf(4, 4, 1, -1, fake, 4, fake, fake, s) == -4
    assert L.bm_sgbtrf(4, 4, 1, 1, fake, 3, fake, fake, s) == -6  # ldab < 2kl+ku+1
    # xgbtrs(trans, n, kl, ku, nrhs, AB, ldab, ipiv, B, ldb, stream)
    assert L.bm_dgbtrs(b"Q", 4, 1, 1, 1, fake, 4, fake, fake, 4, s) == -1
    assert L.bm_dgbtrs(b"N", -1, 1, 1, 1, fake, 4, fake, fake, 4, s) == -2
    assert L.bm_dgbtrs(b"N", 4, 1, 1, -1, fake, 4, fake, fake, 4, s) == -5
    assert L.bm_dgbtrs(b"T", 4, 1, 1, 1, fake, 3, fake, fake, 4, s) == -7
    assert L.bm_dgbtrs(b"N", 4, 1, 1, 1, fake, 4, fake, fake, 3, s) == -10
    # refined batched solve: (count, descs, order, AB, B, X, ipiv, info, AB32, R32, iters,
    # berr, counter, tol, maxit, max_kl, max_ku, stream)
    ok = [fake] * 12

    def ds(count=1, ptrs=None, counter=fake, tol=1e-10, maxit=30, max_kl=2, max_ku=2):
        p = list(ptrs or ok)
        return L.bm_dsgbsv_batched(count, p[0], None, *p[2:11], counter, tol, maxit, max_kl, max_ku, s)

    assert ds(count=-1) == -1
    for arg, idx in ((2, 0), (8, 6), (11, 9), (12, 10)):  # descs, info, iters, berr
        p = list(ok)
        p[idx] = None
        assert ds(ptrs=p) == -arg, arg
    assert ds(counter=None) == -13
    assert ds(tol=float("nan")) == -14
    assert ds(maxit=-1) == -15
    assert ds(max_kl=-1) == -16
    assert ds(max_ku=-1) == -17
    assert ds(count=0, ptrs=[None] * 12) == 0  # an empty batch: nothing to enqueue
    # empty buffers may be NULL (every system with n = 0 or nrhs = 0), not the per-system ones
    p = list(ok)
    p[2] = p[3] = p[4] = p[5] = p[7] = p[8] = None
    assert ds(ptrs=p, counter=None) == -13  # reached the counter check
    # the schedule form checks its schedule as argument 4 and shifts the rest by one
    from importlib import import_module

    Schedule = import_module(bm.__name__ + ".batched").Schedule
    good, bad = Schedule(1, 4, 2, 2, 2, 2), Schedule(1, 3, 2, 2, 2, 2)
    dss = lambda sch, counter=fake, tol=1e-10: L.bm_dsgbsv_batched_sched(
        1, fake, None, ctypes.byref(sch), *([fake] * 9), counter, tol, 30, s)
    assert dss(bad) == -4
    assert dss(good, counter=None) == -14
    assert dss(good, tol=-1.0) == -15


def test_batched_argument_codes_without_gpu(bm):
    """The plain batched entry points report their first illegal argument by position."""
    L = bm._lib.load()
    P = ctypes.c_void_p
    fake, s = P(256), P(0)
    # bm_dgbsv_batched(count, descs, order, AB, ipiv, B, info, counter, max_kl, max_ku, stream)
    b = lambda count=1, descs=fake, info=fake, counter=fake, kl=2, ku=2: L.bm_dgbsv_batched(
        count, descs, None, fake, fake, fake, info, counter, kl, ku, s)
    assert b(count=-1) == -1
    assert b(descs=None) == -2
    assert b(info=None) == -7
    assert b(counter=None) == -8
    assert b(kl=-1) == -9
    assert b(ku=-1) == -10
    assert b(count=0, descs=None, info=None) == 0
    # the schedule form: (count, descs, order, sched, AB, ipiv, B, info, counter, stream)
    from importlib import import_module

    Schedule = import_module(bm.__name__ + ".batched").Schedule
    good, bad = Schedule(1, 4, 2, 2, 2, 2), Schedule(2, 4, 2, 2, 2, 2)  # bad: n_wide > count
    bs = lambda sch, info=fake, counter=fake: L.bm_sgbsv_batched_sched(
        1, fake, None, ctypes.byref(sch), fake, fake, fake, info, counter, s)
    assert bs(bad) == -4
    assert bs(good, info=None) == -8
    assert bs(good, counter=None) == -9
    # the allocation-free form: (count, descs, AB, ipiv, B, info, max_kl, max_ku, stream)
    assert L.bm_dgbsv_batched_noalloc(1, fake, fake, fake, fake, None, 2, 2, s) == -6
    assert L.bm_dgbsv_batched_noalloc(1, fake, fake, fake, fake, fake, -1, 2, s) == -7
    assert L.bm_dgbsv_batched_noalloc(1, fake, fake, fake, fake, fake, 2, -1, s) == -8


def test_product_qr_triangular_and_adjoint_codes_without_gpu(bm):
    """gbmm (src/banded/gbmm.jl:207: C must hold the product's bands), banded QR and its
    Q application, tbsv and the adjoint report their first illegal argument by position."""
    L = bm._lib.load()
    P = ctypes.c_void_p
    f, s = P(256), P(0)
    # gbmm(n, nu, m, Al, Au, Bl, Bu, Cl, Cu, alpha, A, lda, B, ldb, beta, C, ldc, stream)
    g = lambda *a: L.bm_dgbmm(*a[:9], 1.0, f, a[9], f, a[10], 0.0, f, a[11], s)
    assert g(-1, 8, 8, 1, 1, 1, 1, 2, 2, 3, 3, 5) == -1
    assert g(8, 8, 8, 1, -1, 1, 1, 2, 2, 3, 3, 5) == -5
    assert g(8, 8, 8, 1, 1, 1, 1, 1, 2, 3, 3, 5) == -8  # Cl < Al + Bl
    assert g(8, 8, 8, 1, 1, 1, 1, 2, 1, 3, 3, 5) == -9  # Cu < Au + Bu
    assert g(8, 8, 8, 1, 1, 1, 1, 2, 2, 2, 3, 5) == -12
    assert g(8, 8, 8, 1, 1, 1, 1, 2, 2, 3, 2, 5) == -14
    assert g(8, 8, 8, 1, 1, 1, 1, 2, 2, 3, 3, 4) == -17
    # gbqrf(m, n, l, u, AB, ldab, tau, stream); gbqr_lmul(trans, m, n, l, u, AB, ldab, tau,
    # ntau, nrhs, B, ldb, stream); tbsv(uplo, trans, diag, n, k, A, lda, x, incx, stream)
    assert L.bm_dgbqrf(8, 8, -1, 2, f, 6, f, s) == -3
    assert L.bm_dgbqrf(8, 8, 1, 2, f, 3, f, s) == -6
    assert L.bm_dgbqrf(8, 8, 1, 2, f, 6, None, s) == -7
    assert L.bm_dgbqr_lmul(b"X", 8, 8, 1, 2, f, 6, f, 8, 1, f, 8, s) == -1
    assert L.bm_dgbqr_lmul(b"T", 8, 8, 1, 2, f, 6, f, -1, 1, f, 8, s) == -9
    assert L.bm_dgbqr_lmul(b"N", 8, 8, 1, 2, f, 6, f, 8, 1, f, 7, s) == -12
    assert L.bm_dtbsv(b"X", b"N", b"N", 8, 2, f, 3, f, 1, s) == -1
    assert L.bm_dtbsv(b"U", b"X", b"N", 8, 2, f, 3, f, 1, s) == -2
    assert L.bm_dtbsv(b"U", b"N", b"X", 8, 2, f, 3, f, 1, s) == -3
    assert L.bm_dtbsv(b"U", b"N", b"N", 8, 2, f, 2, f, 1, s) == -7
    assert L.bm_dtbsv(b"U", b"T", b"N", 8, 2, f, 3, f, 0, s) == -9
    # adjoint(n, kl, ku, nrhs, LU, ldab, ipiv, X, B, W, grad_B, grad_band, ldg, Xwork, stream)
    adj = lambda n=8, nrhs=1, LU=f, ldab=6, ip=f, X=f, B=f, W=f, gB=f, ldg=4, Xw=f: L.bm_dgbsv_adjoint(
        n, 2, 1, nrhs, LU, ldab, ip, X, B, W, gB, f, ldg, Xw, s)
    assert adj(n=-1) == -1
    assert adj(nrhs=-1) == -4
    assert adj(LU=None) == -5
    assert adj(ldab=5) == -6
    assert adj(ip=None) == -7
    assert adj(X=None, Xw=None) == -8  # X not kept and no workspace to recompute it in
    assert adj(W=None) == -10
    assert adj(gB=None) == -11
    assert adj(ldg=3) == -13
    # nothing to do: the data pointers are not read (an empty call succeeds without a GPU)
    assert adj(n=0, LU=None, ip=None, W=None, gB=None) == 0
    assert adj(nrhs=0, LU=None, ip=None, W=None, gB=None) == 0
