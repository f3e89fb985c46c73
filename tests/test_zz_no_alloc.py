"""fqegpu_apply_noalloc: the H·psi entry point for callers that cannot
allocate device memory (their device memory belongs to another allocator, or
they cannot afford the device synchronisation of cudaMalloc).  It must give
the same sigma as fqegpu_apply, call after call, while using only the static
scratch array compiled into the library.  Collected last (file name) so a
failure here leaves every other test already run."""

import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(lib, norb, na, nb, h1, h2, psi_t, out_t, alpha=1.0, beta=0.0):
    h1c = None if h1 is None else numpy.ascontiguousarray(h1, dtype=numpy.complex128)
    h2c = numpy.ascontiguousarray(h2, dtype=numpy.complex128)
    a, b = complex(alpha), complex(beta)
    p1 = None if h1c is None else h1c.ctypes.data_as(ctypes.c_void_p)
    return lib.fqegpu_apply_noalloc(norb, na, nb, p1,
                                    h2c.ctypes.data_as(ctypes.c_void_p),
                                    ctypes.c_void_p(psi_t.data_ptr()),
                                    ctypes.c_void_p(out_t.data_ptr()),
                                    a.real, a.imag, b.real, b.imag, None)


@pytest.mark.parametrize("norb,na,nb", [(8, 4, 4), (9, 5, 3), (11, 5, 5)])
def test_noalloc_matches_apply_twice(gpu, norb, na, nb):
    import torch
    from fqe_gb300 import _lib, synthetic
    from fqe_gb300.fqe_data import ham_for
    lib = _lib.load()
    h1, h2, rng = synthetic.integrals(norb, norb + 2, 40 + norb)
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data",
              raw_data=synthetic.wavefunction_coeff(d.lena(), d.lenb(), rng))
    ref = d._run_apply(ham_for(d._core, h1, h2), 1.0, 0.25).cpu().numpy()
    for _ in range(2):  # the second call reuses the scratch left by the first
        out = torch.full_like(d.coeff, complex("nan"))
        assert _noalloc(lib, norb, na, nb, h1, h2, d.coeff, out, 1.0, 0.25) == _lib.OK, \
            _lib.last_error()
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        assert numpy.linalg.norm(o - ref) / numpy.linalg.norm(ref) < TOL


@pytest.mark.parametrize("kind", ["complex", "nonsym", "no_h1", "zero"])
def test_noalloc_other_operators(gpu, kind):
    """The uncompressed pair space (complex or non-symmetric integrals,
    P = norb^2), h1 = NULL, and the zero operator (sigma = beta psi), each
    against fqegpu_apply on the same inputs."""
    import torch
    from fqe_gb300 import _lib, synthetic
    from fqe_gb300.fqe_data import ham_for
    lib = _lib.load()
    norb, na, nb = 7, 3, 4
    rng = numpy.random.default_rng(7)
    if kind in ("complex", "nonsym"):
        h1 = rng.normal(size=(norb,) * 2) + 1j * rng.normal(size=(norb,) * 2)
        h2 = rng.normal(size=(norb,) * 4) + 1j * rng.normal(size=(norb,) * 4)
        if kind == "nonsym":
            h1, h2 = h1.real, h2.real
    else:
        h1, h2, _ = synthetic.integrals(norb, norb + 2, 3)
        if kind == "zero":
            h1, h2 = numpy.zeros_like(h1), numpy.zeros_like(h2)
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data",
              raw_data=synthetic.wavefunction_coeff(d.lena(), d.lenb(), rng))
    h1_ref = numpy.zeros((norb, norb)) if kind == "no_h1" else h1
    ref = d._run_apply(ham_for(d._core, h1_ref, h2), 0.5 - 0.25j, 0.75).cpu().numpy()
    out = torch.full_like(d.coeff, complex("nan"))
    rc = _noalloc(lib, norb, na, nb, None if kind == "no_h1" else h1, h2, d.coeff, out,
                  0.5 - 0.25j, 0.75)
    assert rc == _lib.OK, _lib.last_error()
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    assert numpy.linalg.norm(o - ref) / numpy.linalg.norm(ref) < TOL


def test_noalloc_rejects_oversized_sector(gpu):
    import torch
    from fqe_gb300 import _lib
    lib = _lib.load()
    norb, na, nb = 16, 8, 8  # 12870 x 12870: one beta column of D and G is > 64 MiB
    h1 = numpy.eye(norb)
    h2 = numpy.zeros((norb,) * 4)
    h2[0, 1, 1, 0] = 0.1
    buf = torch.zeros(4, dtype=torch.complex128, device="cuda")
    rc = _noalloc(lib, norb, na, nb, h1, h2, buf, buf[2:])
    assert rc == _lib.ERR_UNSUPPORTED
    assert "static scratch" in _lib.last_error()
