"""Wavefunction.save / read on the GPU (wavefunction.py:726-765): a file
written by the reference's own Wavefunction.save loads onto the device with
the reference's coefficients, and this package's files round-trip exactly
(as the reference's test_save_read, tests/wavefunction_test.py:412-441)."""

import numpy
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_read_reference_file(gpu, golden):
    want = golden("saved_wfn")
    wfn = gpu.Wavefunction()
    wfn.read("ref_saved_wfn.pickle", path=GOLDEN)
    assert wfn.norb() == 4
    assert sorted(wfn.sectors()) == [(4, -2), (4, 0), (4, 2)]
    for key in wfn.sectors():
        got = wfn.get_coeff(key).cpu().numpy()
        assert numpy.array_equal(got, want[f"coeff_{key[0]}_{key[1]}"])
    # the loaded wavefunction is usable: an apply runs on it
    h1 = numpy.diag(numpy.arange(1.0, 5.0))
    out = wfn.apply((h1, numpy.zeros((4,) * 4)))
    assert numpy.isfinite(out.get_coeff((4, 0)).cpu().numpy()).all()


def test_save_read_round_trip(gpu, tmp_path):
    import torch
    wfn = gpu.Wavefunction([[6, 0, 6], [6, 2, 6]])
    wfn.set_wfn(strategy="random")
    wfn.save("wfn.pickle", path=str(tmp_path))
    back = gpu.Wavefunction()
    back.read("wfn.pickle", path=str(tmp_path))
    assert back._symmetry_map == wfn._symmetry_map
    assert back._conserved == wfn._conserved
    assert back._conserve_spin == wfn._conserve_spin
    assert back._conserve_number == wfn._conserve_number
    assert back.norb() == wfn.norb()
    for key in wfn.sectors():
        assert torch.equal(back.get_coeff(key), wfn.get_coeff(key))
        assert back.get_coeff(key).is_cuda
