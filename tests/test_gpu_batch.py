"""Batches of applies recorded into one CUDA graph (fqegpu_batch_*): the
replayed results are bit-identical to one-at-a-time applies, including after
the inputs change between launches."""

import numpy
import pytest

pytestmark = pytest.mark.gpu

SECTORS = [(6, 3, 2), (6, 2, 4), (8, 4, 4), (8, 5, 3), (8, 3, 4), (10, 5, 5),
           (10, 6, 4), (7, 0, 3), (9, 4, 5), (6, 3, 3)]


def _setup(gpu):
    from fqe_gb300 import synthetic
    datas, arrays = [], []
    for i, (norb, na, nb) in enumerate(SECTORS):
        h1, h2, psi = synthetic.sector(norb, na, nb, 2 * norb, seed=i)
        d = gpu.FqeData(na, nb, norb)
        d.set_wfn(strategy="from_data", raw_data=psi)
        datas.append(d)
        arrays.append((h1, h2) if i % 4 else (h1,))  # some one-body sectors
    return datas, arrays


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_batch_matches_single_applies(gpu, precision):
    import torch
    from fqe_gb300 import settings
    from fqe_gb300.batch import BatchApply
    datas, arrays = _setup(gpu)
    old = settings.precision
    settings.precision = precision
    try:
        b = BatchApply(datas, arrays, alpha=0.7 - 0.2j, beta=0.25,
                       precision=precision, scratch_limit=8 << 20)
        for rep in range(2):
            if rep:  # new inputs, same buffers
                for d in datas:
                    d.coeff.mul_(-0.5j).add_(0.1)
            b.launch()
            b.check()
            for d, arr, s in zip(datas, arrays, b.sigmas):
                one = d._run_apply(b.hams[datas.index(d)], alpha=0.7 - 0.2j,
                                   beta=0.25)
                torch.cuda.synchronize()
                assert torch.equal(one, s)
    finally:
        settings.precision = old


def test_batch_follows_rebound_coefficients(gpu):
    """FqeData.apply_inplace rebinds `coeff`; the batch keeps the tensors it
    recorded alive and refreshes them from the sectors at launch."""
    import gc
    import torch
    from fqe_gb300 import _lib
    from fqe_gb300.batch import BatchApply
    datas, arrays = _setup(gpu)
    b = BatchApply(datas, arrays, precision="fp64")
    recorded = b.psis[1]
    datas[1].apply_inplace(arrays[1])  # coeff is now a new tensor
    assert datas[1].coeff is not recorded
    gc.collect()
    torch.cuda.empty_cache()
    b.launch()
    b.check()
    one = datas[1]._run_apply(b.hams[1])
    torch.cuda.synchronize()
    assert torch.equal(one, b.sigmas[1])
    # the handles refuse to reallocate or free what the graph holds
    with pytest.raises(ValueError, match="graph"):
        _lib.call("fqegpu_ham_set_scratch_limit", b.hams[0].handle, 1 << 20)
    assert _lib.load().fqegpu_ham_destroy(b.hams[0].handle) == _lib.ERR_INVALID
    ham0 = b.hams[0]
    del b
    gc.collect()
    _lib.call("fqegpu_ham_set_scratch_limit", ham0.handle, 1 << 30)  # released


def test_autotuned_batch_matches_fixed(gpu, oracle):
    """The autotuner (fqe_gb300.autotune) changes the launch shape, or the
    kernels for small sectors, never the result beyond the tensor-core
    tolerance; its choices are cached per sector shape."""
    import torch
    from fqe_gb300 import autotune, synthetic
    from fqe_gb300.batch import BatchApply
    autotune.clear()
    datas, arrays = _setup(gpu)
    arrays = [(a[0], synthetic.integrals(d.norb(), 2 * d.norb(), i)[1])
              for i, (a, d) in enumerate(zip(arrays, datas))]
    b0 = BatchApply(datas, arrays, precision="ozaki")
    b1 = BatchApply(datas, arrays, precision="ozaki", autotune=True)
    for b in (b0, b1):
        b.launch()
        b.check()
    torch.cuda.synchronize()
    assert autotune.cached()
    for d, arr, s0, s1 in zip(datas, arrays, b0.sigmas, b1.sigmas):
        g = oracle.graph(d.norb(), d.nalpha(), d.nbeta())
        want = oracle.apply_spatial12(d.to_numpy(), arr[0], arr[1], g)
        for s in (s0, s1):
            got = s.cpu().numpy()
            assert numpy.linalg.norm(got - want) / numpy.linalg.norm(want) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_batch_repeated_handle_and_overlap(gpu, precision):
    """Through the C ABI: one handle used by three entries (its applies share
    the handle's workspace, so they stay in order on one branch of the graph)
    beside a second handle; results bit-identical to single applies.  A sigma
    that overlaps another entry's psi is refused (the entries may run
    concurrently)."""
    import ctypes
    import torch
    from fqe_gb300 import _lib, synthetic
    from fqe_gb300.fqe_data import _Ham, _ptr
    code = {"fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI}[precision]
    norb, na, nb = 10, 5, 5
    h1, h2, psi = synthetic.sector(norb, na, nb, 20, seed=5)
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)
    e = gpu.FqeData(4, 4, 8)
    g1, g2, psi_e = synthetic.sector(8, 4, 4, 16, seed=6)
    e.set_wfn(strategy="from_data", raw_data=psi_e)
    ha, hb = _Ham(d._core, h1, h2), _Ham(e._core, g1, g2)
    psis = [d.coeff, d.coeff * (0.5 - 1j), e.coeff, d.coeff.conj()]
    hams = [ha, ha, hb, ha]
    sigmas = [torch.empty_like(p) for p in psis]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def create(sig):
        n = len(hams)
        hv = (ctypes.c_void_p * n)(*[h.handle.value for h in hams])
        pv = (ctypes.c_void_p * n)(*[p.data_ptr() for p in psis])
        sv = (ctypes.c_void_p * n)(*[s.data_ptr() for s in sig])
        out = ctypes.c_void_p()
        _lib.call("fqegpu_batch_create", n, hv, pv, sv, 0.3, 0.1, -0.2, 0.0, code, stream,
                  ctypes.byref(out))
        return out

    b = create(sigmas)
    try:
        _lib.call("fqegpu_batch_launch", b, stream)
        _lib.call("fqegpu_batch_check", b, stream)
        for h, p, s in zip(hams, psis, sigmas):
            one = torch.empty_like(p)
            _lib.call("fqegpu_apply", h.handle, _ptr(p), _ptr(one), 0.3, 0.1, -0.2, 0.0, code,
                      stream)
            torch.cuda.synchronize()
            assert torch.equal(one, s)
    finally:
        _lib.load().fqegpu_batch_destroy(b)
    with pytest.raises(ValueError, match="overlaps"):
        create([sigmas[0], sigmas[1], sigmas[2], psis[1]])
