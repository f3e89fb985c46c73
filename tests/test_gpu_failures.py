"""Failure detection, tested without a GPU fault.

The reference exits the process when an allocation fails (safe_malloc,
lib/macros.c:25-46) and has no device waits.  Here every failure becomes a
status code and the context stays usable:

* a bounded wait of the tensor-core kernel runs out: a test hook shortens the
  wait limit and makes the producers of one CTA leave one ring slot unfilled (a
  flag that nothing sets), so the MMA warp's wait gives up; the kernel waits
  for the MMAs it issued, frees its tensor memory and returns; the handle
  reports FQEGPU_ERR_TIMEOUT (TimeoutError) and the next normal apply is
  correct;
* device allocations fail as on an exhausted device (fqegpu_debug_fail_allocs):
  FQEGPU_ERR_NOMEM (MemoryError), and the library works afterwards;
* a coefficient array holding NaN makes the Taylor series stop with
  FQEGPU_ERR_NUMERIC (RuntimeError), as the reference's loop does when its
  norm test cannot be met.
"""

import numpy
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(numpy.linalg.norm(a - b) / numpy.linalg.norm(b))


@pytest.mark.parametrize("skip_slot", [0, 3])
def test_tensor_core_wait_runs_out(gpu, oracle, skip_slot):
    import torch
    from fqe_gb300 import _lib, settings, synthetic
    from fqe_gb300.fqe_data import check_apply, _Ham
    norb, na, nb = 10, 5, 5
    h1, h2, psi = synthetic.sector(norb, na, nb, 20, seed=3)
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)
    ham = _Ham(d._core, h1, h2)  # a private handle: the hook is per handle
    old = settings.precision
    settings.precision = "ozaki"
    try:
        # about 1 ms at 2 GHz: far longer than any wait of a normal apply,
        # far shorter than the default limit
        _lib.call("fqegpu_ham_test_injection", ham.handle, 2_000_000, skip_slot)
        d._run_apply(ham)
        with pytest.raises(TimeoutError, match="bounded wait"):
            check_apply(ham)
        # the error was reported once; the next check is clean
        check_apply(ham)
        _lib.call("fqegpu_ham_test_injection", ham.handle, 0, -1)
        out = d._run_apply(ham)
        check_apply(ham)
        torch.cuda.synchronize()
    finally:
        settings.precision = old
    want = oracle.apply_spatial12(psi, h1, h2, oracle.graph(norb, na, nb))
    assert _rel(out.cpu().numpy(), want) < 1e-10


def test_timeout_reported_by_the_next_apply(gpu):
    import torch
    from fqe_gb300 import _lib, settings, synthetic
    from fqe_gb300.fqe_data import _Ham
    norb, na, nb = 10, 5, 4
    h1, h2, psi = synthetic.sector(norb, na, nb, 20, seed=4)
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)
    ham = _Ham(d._core, h1, h2)
    old = settings.precision
    settings.precision = "ozaki"
    try:
        _lib.call("fqegpu_ham_test_injection", ham.handle, 2_000_000, 0)
        d._run_apply(ham)
        _lib.call("fqegpu_ham_test_injection", ham.handle, 0, -1)
        torch.cuda.synchronize()  # the failed apply has finished
        with pytest.raises(TimeoutError, match="earlier apply"):
            d._run_apply(ham)
        d._run_apply(ham)  # reported once: the handle works again
        _lib.call("fqegpu_ham_check", ham.handle, None)
    finally:
        settings.precision = old


def test_allocation_failure_is_nomem(gpu):
    import torch
    from fqe_gb300 import _lib, synthetic
    from fqe_gb300.fci_graph import FciGraph
    from fqe_gb300.fqe_data import _Ham
    try:
        _lib.call("fqegpu_debug_fail_allocs", 1)
        with pytest.raises(MemoryError):
            FciGraph(3, 4, 9)  # the first table allocation fails
        _lib.call("fqegpu_debug_fail_allocs", 0)
        g = FciGraph(3, 4, 9)
        h1, h2, psi = synthetic.sector(9, 3, 4, 18, seed=5)
        ham = _Ham(g, h1, h2)
        x = torch.from_numpy(psi).cuda()
        y = torch.empty_like(x)
        _lib.call("fqegpu_debug_fail_allocs", 1)
        with pytest.raises(MemoryError):  # the apply's workspace
            _lib.call("fqegpu_apply", ham.handle, x.data_ptr(), y.data_ptr(),
                      1.0, 0.0, 0.0, 0.0, _lib.PREC_FP64, None)
        _lib.call("fqegpu_debug_fail_allocs", 0)
        _lib.call("fqegpu_apply", ham.handle, x.data_ptr(), y.data_ptr(),
                  1.0, 0.0, 0.0, 0.0, _lib.PREC_FP64, None)
        torch.cuda.synchronize()
        assert torch.isfinite(torch.view_as_real(y)).all()
    finally:
        _lib.call("fqegpu_debug_fail_allocs", 0)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_nan_stops_the_taylor_series(gpu, precision):
    from fqe_gb300 import settings, synthetic
    h1, h2, psi = synthetic.sector(8, 4, 4, 16, seed=6)
    psi = psi.copy()
    psi[3, 5] = numpy.nan
    w = gpu.Wavefunction([[8, 0, 8]])
    w.set_wfn(strategy="from_data", raw_data={(8, 0): psi})
    ham = gpu.RestrictedHamiltonian((h1, h2))
    old = settings.precision
    settings.precision = precision
    try:
        with pytest.raises(RuntimeError, match="non-finite"):
            w.apply_generated_unitary(0.05, "taylor", ham, accuracy=1e-12)
    finally:
        settings.precision = old
