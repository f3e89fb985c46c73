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
