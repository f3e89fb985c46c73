"""Block Davidson for the lowest eigenpairs of a restricted Hamiltonian on one
sector (A12 of the path).

The reference (algorithm/davidson.py:140-359) builds its preconditioner
diagonal with one expectation value per determinant (O(N) applies, :159-180),
rebuilds the projected matrix from scratch each iteration and stops on the
change of the eigenvalues (:233).  This driver keeps its entry point and
return values (`davidson_diagonalization(hamiltonian, n_alpha, n_beta,
nroots, guess_vecs)` -> (eigenvalues, eigen-wavefunctions)) and is a
residual-based block Davidson: the diagonal comes from one Slater-Condon pass
(fqegpu_diagonal), H·v from fqegpu_apply (FP64 or tensor-core), inner products
and axpys from libfqegpu (FP64, deterministic), the projected eigenproblem
(<= max_subspace) is solved in FP64 on the host, and a root is converged when
||H x - theta x|| < tol.  The preconditioned residual is
t = m * r / (theta - H_II): m = 1 for the diagonal preconditioner, or the
output of a learned per-determinant correction (fqe_gb300.precond), which can
change the number of iterations but never the converged energy — the residual
decides.
"""

import ctypes
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy
import torch

from . import _lib
from . import settings
from .fci_graph import get_graph
from .fqe_data import FqeData, ham_for, _ptr, _stream
from .hamiltonians import RestrictedHamiltonian
from .wavefunction import Wavefunction


class DiagonalPreconditioner:
    """t = r / (theta - H_II), |theta - H_II| floored (davidson.py:273-280)."""

    name = "diagonal"

    def __init__(self, floor: float = 1.0e-4):
        self.floor = floor

    def __call__(self, r: torch.Tensor, theta: float, diag: torch.Tensor,
                 graph) -> torch.Tensor:
        t = torch.empty_like(r)
        _lib.call("fqegpu_precondition", r.numel(), _ptr(r), _ptr(diag),
                  float(theta), float(self.floor), _ptr(t), _stream())
        return t


class _PlainOf:
    """The plain preconditioner of a learned one (after the residual guard switched)."""

    name = "diagonal"

    def __init__(self, learned):
        self.learned = learned

    def __call__(self, r, theta, diag, graph):
        return self.learned.plain(r, theta, diag, graph)


@dataclass
class DavidsonResult:
    eigenvalues: numpy.ndarray
    vectors: List[torch.Tensor]
    iterations: int
    applies: int
    converged: bool
    residual_history: List[List[float]] = field(default_factory=list)
    seconds: float = 0.0
    fallback_iteration: Optional[int] = None  # learned -> plain switch
    # learned correction vectors that added nothing to the subspace and were
    # replaced by the plain one (before the switch)
    learned_rejected: int = 0


def _vdot(x: torch.Tensor, y: torch.Tensor) -> complex:
    out = (ctypes.c_double * 2)()
    _lib.call("fqegpu_vdot", x.numel(), _ptr(x), _ptr(y), out, _stream())
    return complex(out[0], out[1])


def _axpy(a: complex, x: torch.Tensor, y: torch.Tensor) -> None:
    a = complex(a)
    _lib.call("fqegpu_axpy", x.numel(), a.real, a.imag, _ptr(x), _ptr(y),
              _stream())


def _norm(x: torch.Tensor) -> float:
    out = ctypes.c_double()
    _lib.call("fqegpu_norm2", x.numel(), _ptr(x), ctypes.byref(out), _stream())
    return out.value


def _ptrs(vs: List[torch.Tensor]):
    return (ctypes.c_void_p * len(vs))(*[v.data_ptr() for v in vs])


def _block_vdot(vs: List[torch.Tensor], t: torch.Tensor) -> numpy.ndarray:
    """[<v_i | t>] for all i, one synchronisation."""
    out = numpy.zeros(len(vs), dtype=numpy.complex128)
    for k0 in range(0, len(vs), 64):
        chunk = vs[k0:k0 + 64]
        res = numpy.zeros(2 * len(chunk))
        _lib.call("fqegpu_block_vdot", t.numel(), len(chunk), _ptrs(chunk),
                  _ptr(t), res.ctypes.data_as(ctypes.c_void_p), _stream())
        out[k0:k0 + len(chunk)] = res[0::2] + 1j * res[1::2]
    return out


def _block_axpy(coef, vs: List[torch.Tensor], t: torch.Tensor) -> None:
    """t += sum_i coef[i] v_i, one pass over t."""
    coef = numpy.asarray(coef, dtype=numpy.complex128)
    for k0 in range(0, len(vs), 64):
        chunk = vs[k0:k0 + 64]
        c = numpy.ascontiguousarray(coef[k0:k0 + len(chunk)]).view(numpy.float64)
        _lib.call("fqegpu_block_axpy", t.numel(), len(chunk),
                  c.ctypes.data_as(ctypes.c_void_p), _ptrs(chunk), _ptr(t),
                  _stream())


def _scale(a: complex, x: torch.Tensor) -> None:
    a = complex(a)
    _lib.call("fqegpu_scale", x.numel(), a.real, a.imag, _ptr(x), _stream())


class _Operator:
    """H on one sector: apply, diagonal (both include e_0)."""

    def __init__(self, hamiltonian: RestrictedHamiltonian, nalpha: int,
                 nbeta: int, precision: Optional[str] = None,
                 scratch_limit: Optional[int] = None):
        tensors = hamiltonian.tensors()
        self.norb = hamiltonian.dim()
        self.graph = get_graph(nalpha, nbeta, self.norb)
        self.e0 = complex(hamiltonian.e_0())
        self.ham = ham_for(self.graph, tensors[0],
                           tensors[1] if len(tensors) > 1 else None)
        if scratch_limit is not None:
            # before the first apply: bounds the apply's device workspace
            _lib.call("fqegpu_ham_set_scratch_limit", self.ham.handle,
                      int(scratch_limit))
        self.shape = (self.graph.lena(), self.graph.lenb())
        self.precision = precision
        self.applies = 0
        diag = torch.empty(self.shape, dtype=torch.float64,
                           device=settings.device())
        _lib.call("fqegpu_diagonal", self.ham.handle, _ptr(diag), _stream())
        self.diag = diag + self.e0.real

    def apply(self, v: torch.Tensor) -> torch.Tensor:
        return self.apply_shifted(v, 0.0)

    def check(self) -> None:
        """Waits for the applies so far and raises TimeoutError if a
        tensor-core apply gave up a bounded wait (fqegpu_ham_check)."""
        _lib.call("fqegpu_ham_check", self.ham.handle, _stream())

    def apply_shifted(self, v: torch.Tensor, shift: float) -> torch.Tensor:
        """(H + shift) v."""
        out = torch.empty_like(v)
        code = settings.precision_code() if self.precision is None else {
            "fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI}[self.precision]
        _lib.call("fqegpu_apply", self.ham.handle, _ptr(v), _ptr(out), 1.0,
                  0.0, self.e0.real + shift, self.e0.imag, code, _stream())
        self.applies += 1
        return out


def davidson(hamiltonian: RestrictedHamiltonian, nalpha: int, nbeta: int,
             nroots: int = 1, block: Optional[int] = None, tol: float = 1.0e-6,
             max_subspace: int = 32, max_iter: int = 200,
             guess: Optional[List[torch.Tensor]] = None,
             preconditioner=None, precision: Optional[str] = None,
             verbose: bool = False, callback=None,
             patience: int = 10,
             scratch_limit: Optional[int] = None) -> DavidsonResult:
    """Lowest `nroots` eigenpairs of the sector (nalpha, nbeta).

    `callback(iteration, ritz_vectors, residuals, ritz_values, operator)` is
    called once per iteration before the subspace is expanded (the learned
    preconditioner's training samples are taken there).  `scratch_limit`
    bounds the apply's device workspace (bytes), leaving room for the
    subspace vectors of large sectors.

    A preconditioner with a `plain` method (the learned one) is watched by the
    residual: when the largest residual of the wanted roots has not halved
    over `patience` iterations, the rest of the run uses the plain diagonal
    preconditioner (`fallback_iteration` records when)."""
    t_start = time.time()
    op = _Operator(hamiltonian, nalpha, nbeta, precision, scratch_limit)
    block = max(nroots, block or nroots)
    if max_subspace < 2 * block:
        raise ValueError("max_subspace must hold at least two blocks")
    prec = preconditioner or DiagonalPreconditioner()
    n = op.shape[0] * op.shape[1]
    if nroots > n:
        raise ValueError("Number of roots is incorrectly specified")
    V: List[torch.Tensor] = []
    AV: List[torch.Tensor] = []

    def orthonormal_add(t: torch.Tensor) -> bool:
        # block classical Gram-Schmidt with the Daniel-Gragg-Kaufman-Stewart
        # test: a second pass only when the first removed more than
        # 1 - 1/sqrt(2) of the norm (then the result is orthogonal to working
        # precision either way); each pass is FP64-bound on GB300
        nrm = _norm(t)
        for _ in range(2):
            if not V:
                break
            before = nrm
            _block_axpy(-_block_vdot(V, t), V, t)
            nrm = _norm(t)
            if nrm >= 0.7071067811865476 * before:
                break
        if nrm < 1.0e-10:
            return False
        _scale(1.0 / nrm, t)
        V.append(t)
        AV.append(op.apply(t))
        return True

    # initial block: the lowest diagonal determinants (or the caller's guess)
    if guess:
        for g in guess:
            orthonormal_add(g.clone().to(torch.complex128).reshape(op.shape))
    order = torch.argsort(op.diag.reshape(-1)).cpu().numpy()
    k = 0
    while len(V) < block and k < n:
        e = torch.zeros(op.shape, dtype=torch.complex128, device=op.diag.device)
        e.view(-1)[int(order[k])] = 1.0
        orthonormal_add(e)
        k += 1

    history: List[List[float]] = []
    T = numpy.zeros((0, 0), dtype=numpy.complex128)
    converged = False
    fallback_it = None
    rejected = 0
    best_hist: List[float] = []
    theta = numpy.zeros(nroots)
    X: List[torch.Tensor] = []
    it = 0
    for it in range(1, max_iter + 1):
        op.check()  # the subspace sums below synchronise anyway
        m = len(V)
        Tn = numpy.zeros((m, m), dtype=numpy.complex128)
        Tn[:T.shape[0], :T.shape[1]] = T
        for j in range(T.shape[1], m):   # columns of the new vectors
            Tn[:, j] = _block_vdot(V, AV[j])
        for j in range(T.shape[1]):       # rows of the new vectors (Hermitian)
            Tn[T.shape[0]:, j] = numpy.conj(Tn[j, T.shape[0]:])
        T = 0.5 * (Tn + Tn.conj().T)
        w, y = numpy.linalg.eigh(T)
        X, AX, R, res = [], [], [], []
        for j in range(block):
            x = torch.zeros_like(V[0])
            ax = torch.zeros_like(V[0])
            _block_axpy(y[:, j], V, x)
            _block_axpy(y[:, j], AV, ax)
            r = ax.clone()
            _axpy(-w[j], x, r)
            X.append(x)
            AX.append(ax)
            R.append(r)
            res.append(_norm(r))
        history.append(res[:nroots])
        worst = max(res[:nroots])
        best_hist.append(min(worst, best_hist[-1]) if best_hist else worst)
        if (fallback_it is None and hasattr(prec, "plain")
                and len(best_hist) > patience
                and best_hist[-1] > 0.5 * best_hist[-1 - patience]):
            fallback_it = it
            prec = _PlainOf(prec)
        theta = w[:nroots]
        if callback is not None and not all(rr < tol for rr in res[:nroots]):
            callback(it, X, R, w, op)
        if verbose:
            print(f"davidson iter {it}: theta {w[:nroots]} residual {res[:nroots]}")
        if all(rr < tol for rr in res[:nroots]):
            converged = True
            break
        if m + block > max_subspace:
            # restart on the current Ritz vectors (orthonormal) and their images
            V, AV = list(X), list(AX)
            T = numpy.diag(w[:block]).astype(numpy.complex128)
        added = 0
        for j in range(block):
            if res[j] < tol and j < nroots:
                continue
            t = prec(R[j], float(w[j]), op.diag, op.graph)
            if orthonormal_add(t):
                added += 1
            elif hasattr(prec, "plain"):
                # the learned vector lies in the subspace: plain fallback
                rejected += 1
                if orthonormal_add(prec.plain(R[j], float(w[j]), op.diag,
                                              op.graph)):
                    added += 1
        if added == 0:
            break
    op.check()
    torch.cuda.synchronize()
    return DavidsonResult(fallback_iteration=fallback_it, learned_rejected=rejected,
                          eigenvalues=numpy.array(theta), vectors=X[:nroots],
                          iterations=it, applies=op.applies,
                          converged=converged, residual_history=history,
                          seconds=time.time() - t_start)


def davidsonliu_fqe(hmat: RestrictedHamiltonian, nroots: int, guess_vecs,
                    nele: int, sz: int, norb: int, epsilon: float = 1.0e-8,
                    verbose: bool = False, **kwargs):
    """Reference entry point (algorithm/davidson.py:140-307).  `epsilon` was
    the eigenvalue-change threshold; here the residual tolerance is
    100 * epsilon (the eigenvalue error is of the order of the squared
    residual over the gap).  Same errors: ValueError for a bad root count,
    TypeError when the guesses lie in different sectors."""
    if nroots < 1 or nroots > 2**(hmat.dim() - 1):
        raise ValueError("Number of roots is incorrectly specified")
    sector = list(guess_vecs[0].sectors())[0]
    for gv in guess_vecs:
        if list(gv.sectors())[0] != sector:
            raise TypeError("Sectors don't match for guess vectors")
    if sector != (nele, sz) or hmat.dim() != norb:
        raise ValueError("guess vectors do not match (nele, sz, norb)")
    nalpha, nbeta = (nele + sz) // 2, (nele - sz) // 2
    res = davidson(hmat, nalpha, nbeta, nroots=nroots,
                   guess=[g.get_coeff(sector) for g in guess_vecs],
                   tol=kwargs.pop("tol", 100.0 * epsilon), verbose=verbose,
                   **kwargs)
    return res.eigenvalues, _as_wavefunctions(res.vectors, nele, sz, norb)


def _as_wavefunctions(vectors, nele, sz, norb):
    wfns = []
    for x in vectors:
        w = Wavefunction([[nele, sz, norb]])
        w.set_wfn(strategy="from_data", raw_data={(nele, sz): x})
        wfns.append(w)
    return wfns


def davidson_diagonalization(hamiltonian: RestrictedHamiltonian, n_alpha: int,
                             n_beta: int, nroots: int = 1, guess_vecs=None,
                             **kwargs):
    """Reference entry point (algorithm/davidson.py:310-359): returns
    (eigenvalues, list of eigen-Wavefunctions)."""
    norb = hamiltonian.dim()
    nele, sz = n_alpha + n_beta, n_alpha - n_beta
    guess = None
    if guess_vecs:
        guess = [g.get_coeff((nele, sz)) for g in guess_vecs]
    res = davidson(hamiltonian, n_alpha, n_beta, nroots=nroots, guess=guess,
                   **kwargs)
    return res.eigenvalues, _as_wavefunctions(res.vectors, nele, sz, norb)
