"""Parity of the CUDA path (through the C ABI) with the oracle and the
reference fixtures.  FP64 path: relative error <= 1e-12 (the reference's own
arithmetic differs from ours only in summation order); string tables: bit
exact."""

import ctypes
import math

import numpy
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_OZ = 1e-10


def _rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


def _sector(gpu, norb, na, nb, coeff):
    d = gpu.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=coeff)
    return d


GRAPH_SHAPES = [(0, 0, 0), (1, 1, 0), (1, 0, 1), (2, 1, 1), (4, 2, 2),
                (5, 0, 3), (6, 3, 2), (7, 2, 5), (8, 4, 4), (9, 1, 8),
                (10, 5, 4), (12, 6, 6), (14, 7, 7), (16, 8, 8), (16, 3, 13)]


@pytest.mark.parametrize("norb,na,nb", GRAPH_SHAPES)
def test_graph_bit_exact(gpu, oracle, norb, na, nb):
    g = gpu.FciGraph(na, nb, norb)
    o = oracle.graph(norb, na, nb)
    numpy.testing.assert_array_equal(g._astr, o.astr)
    numpy.testing.assert_array_equal(g._bstr, o.bstr)
    numpy.testing.assert_array_equal(g._dexca, o.dexca)
    numpy.testing.assert_array_equal(g._dexcb, o.dexcb)
    numpy.testing.assert_array_equal(g.z_matrix(0), oracle.z_matrix(norb, na))
    if norb <= 10:
        for i in range(norb):
            for j in range(norb):
                numpy.testing.assert_array_equal(g.alpha_map(i, j), o.alpha_map(i, j))
                numpy.testing.assert_array_equal(g.beta_map(i, j), o.beta_map(i, j))


def test_graph_matches_reference_fixture(gpu, golden):
    gd = golden("graphs")
    for key in [k for k in gd if k.startswith("astr_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        g = gpu.FciGraph(na, nb, norb)
        numpy.testing.assert_array_equal(g._astr, gd["astr_" + tag])
        numpy.testing.assert_array_equal(g._bstr, gd["bstr_" + tag])
        numpy.testing.assert_array_equal(g._dexca, gd["dexca_" + tag])
        numpy.testing.assert_array_equal(g._dexcb, gd["dexcb_" + tag])
        maps = numpy.concatenate([g.alpha_map(i, j).reshape(-1, 3)
                                  for i in range(norb) for j in range(norb)]
                                 ) if norb else numpy.zeros((0, 3), numpy.int32)
        numpy.testing.assert_array_equal(maps, gd["amaps_" + tag])


def test_graph_invalid_arguments(gpu):
    with pytest.raises(ValueError):
        gpu.FciGraph(3, 1, 2)
    with pytest.raises(ValueError):
        gpu.FciGraph(-1, 1, 2)


def test_apply_matches_reference_fixture(gpu, golden):
    gd = golden("apply")
    for key in [k for k in gd if k.startswith("sigma_")]:
        tag = key[6:]
        norb, na, nb = map(int, tag.split("_")[:3])
        tensors = (gd["h1_" + tag],) + ((gd["h2_" + tag],) if "h2_" + tag in gd else ())
        d = _sector(gpu, norb, na, nb, gd["psi_" + tag])
        out = d.apply(tensors).to_numpy()
        assert _rel(out, gd[key]) < TOL_FP64, tag
    # Wavefunction.apply with e_0
    wfn = gpu.Wavefunction([[4, 0, 5]])
    wfn.set_wfn(strategy="from_data", raw_data={(4, 0): gd["e0_psi"]})
    ham = gpu.get_restricted_hamiltonian((gd["e0_h1"], gd["e0_h2"]), e_0=-1.25)
    out = wfn.apply(ham).get_coeff((4, 0)).cpu().numpy()
    assert _rel(out, gd["e0_sigma"]) < TOL_FP64


@pytest.mark.parametrize("norb,na,nb,kind", [
    (6, 3, 3, "real"), (8, 4, 3, "real"), (10, 5, 5, "real"), (10, 2, 7, "real"),
    (7, 3, 4, "complex"), (6, 2, 2, "nonsym"), (9, 0, 4, "real"),
    (8, 8, 2, "real"), (11, 5, 6, "imag"),
])
def test_apply_matches_oracle(gpu, oracle, norb, na, nb, kind):
    rng = numpy.random.default_rng(norb * 100 + na * 10 + nb)
    from fqe_gb300 import synthetic
    if kind in ("real", "imag"):
        h1, h2, _ = synthetic.integrals(norb, norb + 3, norb)
        if kind == "imag":  # -i t h, as the Taylor series applies it
            h1, h2 = -0.07j * h1, -0.07j * h2
    else:
        h1 = rng.normal(size=(norb,) * 2) + 1j * rng.normal(size=(norb,) * 2)
        h2 = rng.normal(size=(norb,) * 4) + 1j * rng.normal(size=(norb,) * 4)
        if kind == "nonsym":
            h1, h2 = h1.real, h2.real
    g = oracle.graph(norb, na, nb)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    ref = oracle.apply_spatial12(psi, h1, h2, g)
    d = _sector(gpu, norb, na, nb, psi)
    out = d.apply((h1, h2)).to_numpy()
    assert _rel(out, ref) < TOL_FP64


def test_apply_streams_beta_blocks(gpu, oracle):
    """A scratch limit below one block forces several beta-column blocks;
    the result must not change."""
    from fqe_gb300 import synthetic
    from fqe_gb300.fqe_data import ham_for, _ptr, _stream
    from fqe_gb300 import _lib
    norb, na, nb = 9, 4, 4
    h1, h2, rng = synthetic.integrals(norb, 12, 5)
    g = oracle.graph(norb, na, nb)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    ref = oracle.apply_spatial12(psi, h1, h2, g)
    d = _sector(gpu, norb, na, nb, psi)
    ham = ham_for(d._core, h1, h2)
    per_col = 2 * ham.npairs * g.lena * 16
    for width in (1, 7, 40):
        _lib.call("fqegpu_ham_set_scratch_limit", ham.handle, per_col * width)
        out = d._run_apply(ham).cpu().numpy()
        assert _rel(out, ref) < TOL_FP64, width
    _lib.call("fqegpu_ham_set_scratch_limit", ham.handle, 1 << 34)


def test_apply_one_body(gpu, oracle):
    rng = numpy.random.default_rng(3)
    for norb, na, nb, cplx in [(6, 3, 2, False), (7, 2, 4, True)]:
        h1 = rng.normal(size=(norb, norb))
        if cplx:
            h1 = h1 + 1j * rng.normal(size=(norb, norb))
        g = oracle.graph(norb, na, nb)
        psi = rng.normal(size=(g.lena, g.lenb)) + 1j * rng.normal(size=(g.lena, g.lenb))
        d = _sector(gpu, norb, na, nb, psi)
        out = d.apply((h1,)).to_numpy()
        assert _rel(out, oracle.apply_spatial1(psi, h1, g)) < TOL_FP64


def test_zero_and_vacuum_sectors(gpu):
    rng = numpy.random.default_rng(4)
    h1 = rng.normal(size=(4, 4))
    h2 = rng.normal(size=(4,) * 4)
    d = _sector(gpu, 4, 0, 0, numpy.array([[0.5 + 0.25j]]))
    assert numpy.abs(d.apply((h1, h2)).to_numpy()).max() == 0.0
    wfn = gpu.Wavefunction([[0, 0, 4]])
    wfn.set_wfn(strategy="from_data", raw_data={(0, 0): numpy.array([[2.0 + 0j]])})
    out = wfn.apply(gpu.get_restricted_hamiltonian((h1, h2), e_0=0.5))
    assert abs(out.get_coeff((0, 0)).item() - 1.0) < 1e-15
    z = _sector(gpu, 4, 2, 1, numpy.ones((6, 4), complex))
    assert numpy.abs(z.apply((h1 * 0, h2 * 0)).to_numpy()).max() == 0.0


def test_diagonal_coulomb_matches_fixture(gpu, golden):
    gd = golden("diagonal_coulomb")
    for key in [k for k in gd if k.startswith("evolve_")]:
        tag = key[7:]
        norb, na, nb = map(int, tag.split("_"))
        psi, v, f = gd["psi_" + tag], gd["v_" + tag], gd["f_" + tag]
        d = _sector(gpu, norb, na, nb, psi)
        ev = d.evolve_diagonal_coulomb(-1j * 0.1 * f, -1j * 0.1 * v).cpu().numpy()
        assert _rel(ev, gd[key]) < TOL_FP64
        ap = d.apply_diagonal_coulomb(f, gd["vns_" + tag]).cpu().numpy()
        assert _rel(ap, gd["apply_" + tag]) < TOL_FP64
        wfn = gpu.Wavefunction([[na + nb, na - nb, norb]])
        wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
        te = wfn.time_evolve(0.1, gpu.get_diagonalcoulomb_hamiltonian(v))
        assert _rel(te.get_coeff((na + nb, na - nb)).cpu().numpy(),
                    gd["time_evolve_" + tag]) < TOL_FP64


def test_diagonal_coulomb_matches_oracle_large(gpu, oracle):
    from fqe_gb300 import synthetic
    norb, na, nb = 12, 6, 5
    g = oracle.graph(norb, na, nb)
    rng = numpy.random.default_rng(12)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    v = synthetic.diagonal_coulomb(norb, 3)
    f = rng.normal(size=norb)
    d = _sector(gpu, norb, na, nb, psi)
    out = d.evolve_diagonal_coulomb(-1j * 0.1 * f, -1j * 0.1 * v).cpu().numpy()
    ref = oracle.evolve_diagonal_coulomb(psi, -1j * 0.1 * f, -1j * 0.1 * v, g)
    assert _rel(out, ref) < TOL_FP64
    # evolve is unitary for real V, f
    assert abs(numpy.linalg.norm(out) - 1.0) < 1e-13


def test_taylor_matches_fixture(gpu, golden):
    gd = golden("taylor")
    for key in [k for k in gd if k.startswith("out_")]:
        tag = key[4:]
        norb, na, nb = map(int, tag.split("_"))
        wfn = gpu.Wavefunction([[na + nb, na - nb, norb]])
        wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): gd["psi_" + tag]})
        ham = gpu.get_restricted_hamiltonian((gd["h1_" + tag], gd["h2_" + tag]))
        out = wfn.apply_generated_unitary(float(gd["t_" + tag]), "taylor", ham,
                                          accuracy=float(gd["acc_" + tag]))
        assert _rel(out.get_coeff((na + nb, na - nb)).cpu().numpy(), gd[key]) < 1e-12


def test_taylor_multi_sector_and_e0(gpu, oracle):
    from fqe_gb300 import synthetic
    norb = 5
    h1, h2, rng = synthetic.integrals(norb, 8, 21)
    wfn = gpu.Wavefunction([[4, 0, norb], [4, 2, norb]])
    data = {}
    for key in wfn.sectors():
        na, nb = gpu.alpha_beta_electrons(*key)
        data[key] = synthetic.wavefunction_coeff(math.comb(norb, na), math.comb(norb, nb), rng)
    wfn.set_wfn(strategy="from_data", raw_data=data)
    ham = gpu.get_restricted_hamiltonian((h1, h2), e_0=0.3)
    out = wfn.apply_generated_unitary(0.1, "taylor", ham, accuracy=1e-13)
    for key in wfn.sectors():
        na, nb = gpu.alpha_beta_electrons(*key)
        g = oracle.graph(norb, na, nb)
        ref, _ = oracle.taylor_evolve(data[key], (h1, h2), 0.3, 0.1, g, accuracy=1e-13)
        # per-sector series stop later or at the same order as the global one
        assert _rel(out.get_coeff(key).cpu().numpy(), ref) < 1e-11


def test_taylor_raises_when_not_converged(gpu):
    from fqe_gb300 import synthetic
    h1, h2, rng = synthetic.integrals(4, 6, 2)
    wfn = gpu.Wavefunction([[4, 0, 4]])
    wfn.set_wfn(strategy="random")
    with pytest.raises(RuntimeError):
        wfn.apply_generated_unitary(50.0, "taylor",
                                    gpu.get_restricted_hamiltonian((h1, h2)),
                                    expansion=3)


def test_dvec_matches_fixture(gpu, golden):
    gd = golden("dvec")
    for key in [k for k in gd if k.startswith("dvec_")]:
        tag = key[5:]
        norb, na, nb = map(int, tag.split("_"))
        d = _sector(gpu, norb, na, nb, gd["psi_" + tag])
        dv = d.calculate_dvec_spatial()
        numpy.testing.assert_allclose(dv.cpu().numpy(), gd[key], rtol=0, atol=1e-15)
        co = d._calculate_coeff_spatial_with_dvec(dv).cpu().numpy()
        assert _rel(co, gd["coeff_" + tag]) < 1e-14


def test_vector_ops(gpu):
    import torch
    rng = numpy.random.default_rng(7)
    a = rng.normal(size=(70, 56)) + 1j * rng.normal(size=(70, 56))
    b = rng.normal(size=(70, 56)) + 1j * rng.normal(size=(70, 56))
    x = _sector(gpu, 8, 4, 3, a)
    y = _sector(gpu, 8, 4, 3, b)
    assert abs(x.norm() - numpy.linalg.norm(a)) < 1e-12
    assert abs(x.vdot(y) - numpy.vdot(a, b)) < 1e-10
    y.ax_plus_y(0.3 - 0.2j, x)
    assert _rel(y.to_numpy(), b + (0.3 - 0.2j) * a) < 1e-15
    x.scale(1.5j)
    assert _rel(x.to_numpy(), 1.5j * a) < 1e-15
    # deterministic reductions
    assert x.norm() == x.norm()


def test_diagonal_energies(gpu, oracle):
    from fqe_gb300 import synthetic
    for norb, na, nb in [(5, 2, 3), (6, 3, 3)]:
        h1, h2, _ = synthetic.integrals(norb, 7, norb)
        g = oracle.graph(norb, na, nb)
        ref = oracle.diagonal_energies(h1, h2, g).real
        d = gpu.FqeData(na, nb, norb)
        out = d.diagonal_energies(h1, h2).cpu().numpy()
        numpy.testing.assert_allclose(out, ref, rtol=0, atol=1e-11)


def test_apply_host_entry_point(gpu, oracle):
    """fqegpu_apply_host: the call a ctypes binding in the reference's FqeData
    would make, with numpy (host) buffers."""
    from fqe_gb300 import synthetic, _lib
    from fqe_gb300.fqe_data import ham_for
    norb, na, nb = 8, 4, 4
    h1, h2, rng = synthetic.integrals(norb, 16, 0)
    g = oracle.graph(norb, na, nb)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    graph = gpu.FciGraph(na, nb, norb)
    ham = ham_for(graph, h1, h2)
    out = numpy.zeros_like(psi)
    _lib.call("fqegpu_apply_host", ham.handle, psi.ctypes.data_as(ctypes.c_void_p),
              out.ctypes.data_as(ctypes.c_void_p), 1.0, 0.0, 0.0, 0.0, 0)
    assert _rel(out, oracle.apply_spatial12(psi, h1, h2, g)) < TOL_FP64


@pytest.mark.parametrize("blocked", [False, True])
def test_apply_host_tensor_cores(gpu, oracle, blocked):
    """fqegpu_apply_host on the tensor-core path, whose last scatter runs in
    row chunks with sigma copied out behind it (pageable numpy buffers), in
    one block and in beta-column blocks (a small scratch limit); twice, so
    the handle's copy stream is reused."""
    from fqe_gb300 import synthetic, _lib
    from fqe_gb300.fqe_data import _Ham
    norb, na, nb = 10, 5, 5
    h1, h2, rng = synthetic.integrals(norb, 20, 3)
    g = oracle.graph(norb, na, nb)
    psi = synthetic.wavefunction_coeff(g.lena, g.lenb, rng)
    ham = _Ham(gpu.FciGraph(na, nb, norb), h1, h2)
    if blocked:
        _lib.call("fqegpu_ham_set_scratch_limit", ham.handle, 8 << 20)  # 32-column blocks
    want = 0.5 * oracle.apply_spatial12(psi, h1, h2, g) - 0.25j * psi
    for _ in range(2):
        out = numpy.full_like(psi, numpy.nan)
        _lib.call("fqegpu_apply_host", ham.handle, psi.ctypes.data_as(ctypes.c_void_p),
                  out.ctypes.data_as(ctypes.c_void_p), 0.5, 0.0, 0.0, -0.25, 1)
        assert _rel(out, want) < TOL_OZ


def test_apply_rejects_aliasing_and_bad_precision(gpu):
    from fqe_gb300 import synthetic, _lib
    from fqe_gb300.fqe_data import ham_for, _ptr
    h1, h2, rng = synthetic.integrals(4, 5, 1)
    d = gpu.FqeData(2, 2, 4)
    ham = ham_for(d._core, h1, h2)
    with pytest.raises(ValueError):
        _lib.call("fqegpu_apply", ham.handle, _ptr(d.coeff), _ptr(d.coeff),
                  1.0, 0.0, 0.0, 0.0, 0, None)
    out = d.coeff.clone()
    with pytest.raises(ValueError):
        _lib.call("fqegpu_apply", ham.handle, _ptr(d.coeff), _ptr(out),
                  1.0, 0.0, 0.0, 0.0, 17, None)


def test_apply_deterministic(gpu):
    from fqe_gb300 import synthetic
    h1, h2, rng = synthetic.integrals(10, 12, 2)
    psi = synthetic.wavefunction_coeff(252, 210, rng)
    d = _sector(gpu, 10, 5, 4, psi)
    a = d.apply((h1, h2)).to_numpy()
    b = d.apply((h1, h2)).to_numpy()
    assert numpy.array_equal(a, b)


def test_reference_wavefunction_pickles(gpu, golden):
    # the reference's own Wavefunction.apply golden data (restricted
    # Hamiltonians with e_0, diagonal Coulomb), every sector, FP64 path
    gd = golden("wfn_pickles")
    for key in [k for k in gd if k.startswith("out_")]:
        name, kind, na, nb = key[4:].rsplit("_", 3)
        tag = f"{name}_{kind}"
        norb, na, nb = int(gd["norb_" + tag]), int(na), int(nb)
        psi = gd[f"psi_{tag}_{na}_{nb}"]
        e0 = complex(gd["e0_" + tag])
        want = gd[key]
        if kind == "array":
            wfn = gpu.Wavefunction([[na + nb, na - nb, norb]])
            wfn.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
            ham = gpu.get_restricted_hamiltonian((gd["t0_" + tag], gd["t1_" + tag]),
                                                 e_0=e0)
            out = wfn.apply(ham).get_coeff((na + nb, na - nb)).cpu().numpy()
        else:
            d = _sector(gpu, norb, na, nb, psi)
            out = d.apply_diagonal_coulomb(gd["diag_" + tag],
                                           gd["vij_" + tag]).cpu().numpy()
            if abs(e0) > 1e-15:
                out = out + e0 * psi
        assert numpy.abs(out - want).max() <= TOL_FP64 * max(1.0, numpy.abs(want).max())
