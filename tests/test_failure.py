"""Failure detection without a GPU fault.

* The bounded in-kernel waits give up after their poll limit, record the timeout bit in
  the device status word (bm_device_status) and return; the context stays usable.  The
  wait that runs out is on an mbarrier phase that nothing completes, with a short
  host-set limit (bm_wait_selftest), through the same helper the streaming kernels use.
* The batched kernels check every descriptor on the device before they touch its
  system: an illegal field, or a band wider than the bounds the launch's shared memory
  was sized for, gives info[s] = -(field number) and the system is skipped, while every
  other system of the batch is solved exactly as in a clean batch.  The planted faults
  are host-written descriptor values that the kernels' own checks turn into errors.
"""
import ctypes

import numpy as np
import pytest
import torch


def test_wait_selftest_argument_codes(bm):
    L = bm._lib.load()
    fake = ctypes.c_void_p(256)  # never dereferenced: the calls stop at an argument check
    assert L.bm_wait_selftest(0, fake, None) == -1
    assert L.bm_wait_selftest((1 << 26) + 1, fake, None) == -1
    assert L.bm_wait_selftest(100, None, None) == -2


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.gpu
def test_bounded_wait_times_out_and_reports(bm, gpu):
    L = bm._lib.load()
    st = ctypes.c_int(-1)
    assert L.bm_device_status(ctypes.byref(st), 1, _stream()) == 0  # start clear
    done = torch.zeros(1, dtype=torch.int32, device=gpu)
    assert L.bm_wait_selftest(1 << 12, ctypes.c_void_p(done.data_ptr()), _stream()) == 0, L.bm_last_error()
    torch.cuda.synchronize()
    assert int(done.item()) == 1  # the kernel left its wait and returned
    assert L.bm_device_status(ctypes.byref(st), 1, _stream()) == 0
    assert st.value & 1, "the timeout bit is not set"
    # the context still works, and the status word was cleared by the read above
    A = bm.brandn(torch.float64, 300, 300, 2, 3, device=gpu)
    x = torch.randn(300, dtype=torch.float64, device=gpu)
    y = bm.mul(A, x)
    torch.cuda.synchronize()
    assert torch.isfinite(y).all()
    assert L.bm_device_status(ctypes.byref(st), 0, _stream()) == 0
    assert st.value == 0


def _make(bm, gpu, rng, count, kl_hi, ku_hi, n_hi=600):
    n = rng.integers(20, n_hi, count)
    kl = rng.integers(0, kl_hi + 1, count)
    ku = rng.integers(0, ku_hi + 1, count)
    nrhs = rng.integers(1, 4, count)
    kl[0], ku[0] = kl_hi, ku_hi  # the bounds are reached
    batch = bm.BandedBatch(n, kl, ku, nrhs, torch.float64, gpu)
    bands = [torch.from_numpy(rng.standard_normal((kl[s] + ku[s] + 1, n[s]))) for s in range(count)]
    for s in range(count):
        bands[s][ku[s], :] += 2.0 * (kl[s] + ku[s]) + 1.0
    rhs = [torch.from_numpy(rng.standard_normal((n[s], nrhs[s]))) for s in range(count)]
    return batch, bands, rhs


def _load(batch, bands, rhs):
    batch.AB.zero_()
    for s in range(batch.count):
        batch.matrix_band(s).copy_(bands[s])
        batch.rhs(s).copy_(rhs[s])
    batch.ipiv.fill_(-7)
    batch.info.fill_(-77)


def _plant(batch):
    """Bad descriptors on the device: system 2's kl above the launch bound, system 3's
    ldab too small, system 4's band offset negative; and system 5 is not in the order
    list (its entry replaced by an index outside the batch).  Returns
    {system: expected info} and the skipped system."""
    d = batch.descs
    d[2, 1] = batch.max_kl + 3
    d[3, 5] = 1
    d[4, 4] = -8
    k = int((batch.order == 5).nonzero()[0, 0])
    batch.order[k] = batch.count + 1000
    return {2: -2, 3: -6, 4: -5}, 5


def _check(batch, ref, bad, skipped, x_of):
    info = batch.info.cpu().numpy()
    for s, code in bad.items():
        assert info[s] == code, (s, info[s])
    assert info[skipped] == -77
    for s in range(batch.count):
        if s in bad or s == skipped:
            continue
        assert info[s] == ref["info"][s], s
        assert np.array_equal(x_of(s), ref["x"][s]), s


@pytest.mark.gpu
@pytest.mark.parametrize("sched", [None, (4, 12)])
def test_plain_batched_rejects_bad_descriptors(bm, gpu, sched):
    rng = np.random.default_rng(11)
    batch, bands, rhs = _make(bm, gpu, rng, 40, 20, 14)
    if sched:
        batch.set_schedule(*sched)
    _load(batch, bands, rhs)
    batch.factor_solve()
    torch.cuda.synchronize()
    ref = {"info": batch.info.cpu().numpy(), "x": [batch.rhs(s).cpu().numpy() for s in range(batch.count)]}
    _load(batch, bands, rhs)
    bad, skipped = _plant(batch)
    batch.factor_solve()
    torch.cuda.synchronize()
    _check(batch, ref, bad, skipped, lambda s: batch.rhs(s).cpu().numpy())
    for s in list(bad) + [skipped]:  # a rejected or skipped system's data is untouched
        assert torch.equal(batch.rhs(s).cpu(), rhs[s])


@pytest.mark.gpu
def test_noalloc_batched_rejects_bad_descriptors(bm, gpu):
    rng = np.random.default_rng(12)
    batch, bands, rhs = _make(bm, gpu, rng, 40, 20, 14)
    _load(batch, bands, rhs)
    batch.factor_solve()
    torch.cuda.synchronize()
    ref = {"info": batch.info.cpu().numpy(), "x": [batch.rhs(s).cpu().numpy() for s in range(batch.count)]}
    _load(batch, bands, rhs)
    bad, _ = _plant(batch)  # the allocation-free solve builds its own order
    L = bm._lib.load()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    st = L.bm_dgbsv_batched_noalloc(batch.count, p(batch.descs), p(batch.AB), p(batch.ipiv), p(batch.B),
                                    p(batch.info), batch.max_kl, batch.max_ku, _stream())
    assert st == 0, L.bm_last_error()
    torch.cuda.synchronize()
    info = batch.info.cpu().numpy()
    for s in range(batch.count):
        if s in bad:
            assert info[s] == bad[s]
        else:
            assert info[s] == ref["info"][s]
            assert np.array_equal(batch.rhs(s).cpu().numpy(), ref["x"][s]), s


@pytest.mark.gpu
@pytest.mark.parametrize("kl_hi,ku_hi", [(20, 14), (84, 10)])  # blocked FP32 path; group path (kl > 80)
def test_refined_batched_rejects_bad_descriptors(bm, gpu, kl_hi, ku_hi):
    rng = np.random.default_rng(13)
    batch, bands, rhs = _make(bm, gpu, rng, 24, kl_hi, ku_hi, n_hi=400)
    _load(batch, bands, rhs)
    batch.solve_mixed(1e-12, 30)
    torch.cuda.synchronize()
    ref = {"info": batch.info.cpu().numpy(), "x": [batch.solution(s).cpu().numpy() for s in range(batch.count)]}
    _load(batch, bands, rhs)
    batch.X.fill_(0.5)
    bad, skipped = _plant(batch)
    batch.solve_mixed(1e-12, 30)
    torch.cuda.synchronize()
    _check(batch, ref, bad, skipped, lambda s: batch.solution(s).cpu().numpy())
    its = batch.iters.cpu().numpy()
    for s in bad:  # neither factored nor refined; X untouched
        assert its[s] == 0
        assert (batch.solution(s) == 0.5).all()
