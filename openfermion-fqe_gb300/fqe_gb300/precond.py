"""Learned Davidson preconditioner (A12): a per-determinant MLP that corrects
the diagonal preconditioner, trained on exact correction-equation solutions.

No counterpart in the reference, whose Davidson (algorithm/davidson.py:
273-280) uses t = r / (theta - H_II).  Here t_I = m_I r_I / (theta - H_II)
with m_I = 1 + tanh(MLP(features_I)) in (0, 2); the network is 34 -> 64 ->
64 -> 1 with bfloat16 weights, evaluated by a hand-written inference kernel
fused with the preconditioning (fqegpu_mlp_precondition) and trained by
hand-written forward/backward kernels and Adam (fqegpu_mlp_loss_grad,
fqegpu_mlp_adam).  Training samples come from the method itself: Davidson
runs on small sectors, and at each iteration the Jacobi-Davidson correction
equation
    (1 - x x^H)(H - theta)(1 - x x^H) a = -r,   a _|_ x
is solved by MINRES with GPU applies; the network learns to turn the
diagonal correction u = r / (theta - H_II) into a vector as parallel as
possible to a outside x (the loss is one minus the squared cosine).

The plain preconditioner is the fallback: for norb > 16, and whenever the
learned vector adds nothing new to the subspace.  The Davidson residual
decides convergence either way, so the network changes iteration counts and
never the converged energy.
"""

import ctypes
import math
import os
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy
import torch

from . import _lib
from .fqe_data import _ptr, _stream

NPARAM = 6465
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                               "data", "precond_mlp.npz")


def init_params(seed: int = 0) -> numpy.ndarray:
    """He-initialised hidden layers, zero output layer: m = 1 (the plain
    preconditioner) until training moves the output layer."""
    rng = numpy.random.default_rng(seed)
    w1 = rng.normal(0.0, math.sqrt(2.0 / 34), (64, 34))
    w2 = rng.normal(0.0, math.sqrt(2.0 / 64), (64, 64))
    return numpy.concatenate([w1.ravel(), numpy.zeros(64), w2.ravel(),
                              numpy.zeros(64), numpy.zeros(64),
                              numpy.zeros(1)]).astype(numpy.float32)


def _diag_stats(diag: torch.Tensor):
    """(population standard deviation, minimum) of H_II."""
    return float(diag.std(correction=0)), float(diag.min())


class LearnedPreconditioner:
    """Callable with the DiagonalPreconditioner signature
    (r, theta, diag, graph) -> t; owns one fqegpu_mlp handle."""

    name = "learned"

    def __init__(self, params: Optional[numpy.ndarray] = None,
                 floor: float = 1.0e-4):
        if int(_lib.load().fqegpu_mlp_nparams()) != NPARAM:
            raise RuntimeError("libfqegpu.so parameter layout mismatch")
        h = ctypes.c_void_p()
        _lib.call("fqegpu_mlp_create", ctypes.byref(h))
        self.handle = h
        self.floor = floor
        self._stats_key = None
        self._stats = None
        self.set_params(numpy.zeros(NPARAM, numpy.float32)
                        if params is None else params)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.fqegpu_mlp_destroy(h)
            self.handle = None

    # -- parameters -----------------------------------------------------------
    def set_params(self, params: numpy.ndarray) -> None:
        p = numpy.ascontiguousarray(params, dtype=numpy.float32)
        if p.shape != (NPARAM,):
            raise ValueError(f"expected {NPARAM} parameters")
        _lib.call("fqegpu_mlp_set_params", self.handle,
                  p.ctypes.data_as(ctypes.c_void_p), NPARAM)

    def params(self) -> numpy.ndarray:
        p = numpy.empty(NPARAM, numpy.float32)
        _lib.call("fqegpu_mlp_get_params", self.handle,
                  p.ctypes.data_as(ctypes.c_void_p), NPARAM)
        return p

    def grad(self) -> numpy.ndarray:
        g = numpy.empty(NPARAM, numpy.float32)
        _lib.call("fqegpu_mlp_get_grad", self.handle,
                  g.ctypes.data_as(ctypes.c_void_p), NPARAM)
        return g

    def save(self, path: str, **meta) -> None:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        numpy.savez(path, params=self.params(),
                    meta=numpy.array(repr(meta)))

    @classmethod
    def load(cls, path: str = DEFAULT_WEIGHTS, **kw) -> "LearnedPreconditioner":
        with numpy.load(path) as d:
            return cls(d["params"], **kw)

    # -- inference ------------------------------------------------------------
    def stats(self, diag: torch.Tensor):
        key = (diag.data_ptr(), diag.numel())
        if key != self._stats_key:
            self._stats_key, self._stats = key, _diag_stats(diag)
        return self._stats

    def __call__(self, r: torch.Tensor, theta: float, diag: torch.Tensor,
                 graph) -> torch.Tensor:
        t = torch.empty_like(r)
        if graph.norb() > 16:
            _lib.call("fqegpu_precondition", r.numel(), _ptr(r), _ptr(diag),
                      float(theta), float(self.floor), _ptr(t), _stream())
            return t
        scale, emin = self.stats(diag)
        _lib.call("fqegpu_mlp_precondition", self.handle, graph.handle,
                  _ptr(r), _ptr(diag), float(theta), scale, emin,
                  float(self.floor), _ptr(t), _stream())
        return t

    def plain(self, r, theta, diag, graph):
        """The plain diagonal preconditioner (the fallback)."""
        t = torch.empty_like(r)
        _lib.call("fqegpu_precondition", r.numel(), _ptr(r), _ptr(diag),
                  float(theta), float(self.floor), _ptr(t), _stream())
        return t

    def multiplier(self, theta: float, diag: torch.Tensor, graph) -> torch.Tensor:
        m = torch.empty(diag.shape, dtype=torch.float32, device=diag.device)
        scale, emin = self.stats(diag)
        _lib.call("fqegpu_mlp_multiplier", self.handle, graph.handle,
                  _ptr(diag), float(theta), scale, emin, _ptr(m), _stream())
        return m

    # -- training -------------------------------------------------------------
    def loss_grad(self, s: "CorrectionSample", accumulate: bool = False) -> float:
        out = ctypes.c_double()
        _lib.call("fqegpu_mlp_loss_grad", self.handle, s.graph.handle,
                  _ptr(s.u), _ptr(s.x), _ptr(s.a), _ptr(s.diag),
                  float(s.theta), s.scale, s.emin, int(accumulate),
                  ctypes.byref(out), _stream())
        return out.value

    def adam(self, lr: float, grad_scale: float = 1.0, beta1: float = 0.9,
             beta2: float = 0.999, eps: float = 1.0e-8) -> None:
        _lib.call("fqegpu_mlp_adam", self.handle, float(lr), float(beta1),
                  float(beta2), float(eps), float(grad_scale), _stream())


@dataclass
class CorrectionSample:
    """One Davidson iteration's correction equation, resident on the GPU."""
    graph: object
    diag: torch.Tensor
    theta: float
    u: torch.Tensor        # r / (theta - H_II), floored
    x: torch.Tensor        # Ritz vector (normalised)
    a: torch.Tensor        # correction-equation solution, orthogonal to x
    scale: float
    emin: float
    solve_residual: float = 0.0
    meta: dict = field(default_factory=dict)


def _vdot(x, y) -> complex:
    out = (ctypes.c_double * 2)()
    _lib.call("fqegpu_vdot", x.numel(), _ptr(x), _ptr(y), out, _stream())
    return complex(out[0], out[1])


def _axpy(a, x, y) -> None:
    a = complex(a)
    _lib.call("fqegpu_axpy", x.numel(), a.real, a.imag, _ptr(x), _ptr(y),
              _stream())


def _scale(a, x) -> None:
    a = complex(a)
    _lib.call("fqegpu_scale", x.numel(), a.real, a.imag, _ptr(x), _stream())


def _norm(x) -> float:
    out = ctypes.c_double()
    _lib.call("fqegpu_norm2", x.numel(), _ptr(x), ctypes.byref(out),
              _stream())
    return out.value


def minres(apply_a, b: torch.Tensor, tol: float = 1.0e-8,
           maxiter: int = 300):
    """MINRES (Paige & Saunders 1975) for a Hermitian operator, all vector
    arithmetic through libfqegpu.  Returns (solution, relative residual
    estimate, iterations)."""
    x = torch.zeros_like(b)
    beta1 = _norm(b)
    if beta1 == 0.0:
        return x, 0.0, 0
    r1 = b.clone()
    r2 = b.clone()
    y = b.clone()
    w = torch.zeros_like(b)
    w2 = torch.zeros_like(b)
    oldb, beta, dbar, epsln = 0.0, beta1, 0.0, 0.0
    phibar, cs, sn = beta1, -1.0, 0.0
    itn = 0
    for itn in range(1, maxiter + 1):
        v = y.clone()
        _scale(1.0 / beta, v)
        y = apply_a(v)
        if itn >= 2:
            _axpy(-beta / oldb, r1, y)
        alfa = _vdot(v, y).real
        _axpy(-alfa / beta, r2, y)
        r1, r2 = r2, y.clone()
        oldb, beta = beta, _norm(r2)
        oldeps = epsln
        delta = cs * dbar + sn * alfa
        gbar = sn * dbar - cs * alfa
        epsln = sn * beta
        dbar = -cs * beta
        gamma = max(math.hypot(gbar, beta), 1e-300)
        cs, sn = gbar / gamma, beta / gamma
        phi = cs * phibar
        phibar = sn * phibar
        w1, w2 = w2, w
        w = v.clone()
        _axpy(-oldeps, w1, w)
        _axpy(-delta, w2, w)
        _scale(1.0 / gamma, w)
        _axpy(phi, w, x)
        if phibar / beta1 < tol or beta == 0.0:
            break
    return x, phibar / beta1, itn


def correction_sampler(store: List[CorrectionSample], every: int = 1,
                       tol: float = 1.0e-8, maxiter: int = 300,
                       max_samples: Optional[int] = None, meta=None):
    """Davidson callback that solves the correction equation of root 0 at
    every `every`-th iteration and appends a CorrectionSample to `store`."""

    def cb(it, X, R, w, op, prec_floor=1.0e-4):
        if max_samples is not None and len(store) >= max_samples:
            return
        if (it - 1) % every:
            return
        x, r, theta = X[0], R[0], float(w[0])

        def proj(v):
            _axpy(-_vdot(x, v), x, v)
            return v

        def apply_a(v):
            p = proj(v.clone())
            out = op.apply_shifted(p, -theta)
            return proj(out)

        rhs = r.clone()
        _scale(-1.0, rhs)
        proj(rhs)
        a, res, _ = minres(apply_a, rhs, tol=tol, maxiter=maxiter)
        proj(a)
        u = torch.empty_like(r)
        _lib.call("fqegpu_precondition", r.numel(), _ptr(r), _ptr(op.diag),
                  theta, prec_floor, _ptr(u), _stream())
        scale, emin = _diag_stats(op.diag)
        store.append(CorrectionSample(
            graph=op.graph, diag=op.diag, theta=theta, u=u, x=x.clone(), a=a,
            scale=scale, emin=emin, solve_residual=res,
            meta=dict(meta or {}, iteration=it)))

    return cb


def mean_loss(pre: LearnedPreconditioner, samples) -> float:
    return float(numpy.mean([pre.loss_grad(s) for s in samples]))


def train(pre: LearnedPreconditioner, samples: List[CorrectionSample],
          epochs: int = 30, lr: float = 1.0e-3, batch: int = 4, seed: int = 0,
          log=None) -> List[float]:
    """Adam over minibatches of samples (gradients summed by the loss kernels
    with accumulate=1, scaled by 1/batch).  Returns the mean loss per epoch."""
    rng = numpy.random.default_rng(seed)
    history = []
    for ep in range(epochs):
        order = rng.permutation(len(samples))
        tot = 0.0
        for k in range(0, len(order), batch):
            idx = order[k:k + batch]
            for j, i in enumerate(idx):
                tot += pre.loss_grad(samples[i], accumulate=j > 0)
            pre.adam(lr, grad_scale=1.0 / len(idx))
        history.append(tot / len(samples))
        if log:
            log(f"epoch {ep}: mean loss {history[-1]:.6f}")
    return history
