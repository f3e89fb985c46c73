"""ORACLE — test infrastructure only (never imported by the GPU product).

CPU FP64 restatement of the learned Davidson preconditioner: determinant
features, the 34 -> 64 -> 64 -> 1 network, the correction-equation loss and its
analytic gradient.  The reference has no learned preconditioner (its Davidson,
algorithm/davidson.py:273-280, uses the plain 1 / (theta - H_II)); this file
is the specification the CUDA kernels (csrc/mlp.cu) are checked against, and
its own gradient is pinned by central finite differences in
tests/test_mlp_oracle.py.

Parameter vector (float32 master copy, 6465 entries, in this order):
    W1[64][34], b1[64], W2[64][64], b2[64], w3[64], b3
The forward pass uses the weights rounded to bfloat16 (round to nearest
even); activations and sums are float32 on the GPU and float64 here.

Features of determinant I = (alpha string a, beta string b), theta = Ritz value:
    f0 = (H_II - theta) / s,   f1 = (theta - min_J H_JJ) / s
    f2..f17  = alpha occupation of slots 0..15, f18..f33 = beta slots 0..15,
where slot k holds orbital k - 8 + n_spin (the Fermi level of the spin sits
between slots 7 and 8); slots below orbital 0 read 1 (a filled core), slots
beyond the last orbital read 0.  s is the standard deviation of H_II over
the sector.

Network: z1 = W1 f + b1, h1 = relu(z1), z2 = W2 h1 + b2, h2 = relu(z2),
z3 = w3 . h2 + b3, m = 1 + tanh(z3).  Preconditioned residual
t_I = m_I r_I / d_I with d_I = theta - H_II, |d_I| >= floor.

Loss of one sample (u = r / d, x = Ritz vector, a = exact correction, a _|_ x):
    w = m * u,  v = w - x (x^H w),  L = 1 - |a^H v|^2 / (|a|^2 |v|^2).
"""

import numpy

NIN, NH = 34, 64
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
         ("w3", (NH,)), ("b3", (1,))]
NPARAM = sum(int(numpy.prod(s)) for _, s in SIZES)


def unpack(p):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(numpy.prod(shape))
        out[name] = numpy.asarray(p[k:k + n], dtype=numpy.float64).reshape(shape)
        k += n
    return out


def bf16_round(p):
    """float32 -> nearest-even bfloat16, returned as float32 values."""
    u = numpy.asarray(p, dtype=numpy.float32).view(numpy.uint32).astype(numpy.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(numpy.uint32).view(numpy.float32)


def slot_bits(strings, norb, nele):
    """[len, 16] Fermi-aligned occupation slots of bit strings."""
    out = numpy.zeros((len(strings), 16))
    for k in range(16):
        orb = k - 8 + nele
        if orb < 0:
            out[:, k] = 1.0
        elif orb < norb:
            out[:, k] = [(int(s) >> orb) & 1 for s in strings]
    return out


def features(diag, theta, astr, bstr, norb, nalpha, nbeta, scale, emin):
    """[lena * lenb, 34] feature matrix (determinant I = a * lenb + b)."""
    la, lb = len(astr), len(bstr)
    A = slot_bits(astr, norb, nalpha)
    B = slot_bits(bstr, norb, nbeta)
    f = numpy.empty((la * lb, NIN))
    f[:, 0] = (numpy.asarray(diag, dtype=numpy.float64).ravel() - theta) / scale
    f[:, 1] = (theta - emin) / scale
    f[:, 2:18] = numpy.repeat(A, lb, axis=0)
    f[:, 18:34] = numpy.tile(B, (la, 1))
    return f


def forward(params, f, cache=False, rounding=True):
    w = unpack(bf16_round(params) if rounding else params)
    z1 = f @ w["W1"].T + w["b1"]
    h1 = numpy.maximum(z1, 0.0)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = numpy.maximum(z2, 0.0)
    z3 = h2 @ w["w3"] + w["b3"][0]
    m = 1.0 + numpy.tanh(z3)
    if cache:
        return m, (w, f, z1, h1, z2, h2)
    return m


def floored(diag, theta, floor):
    d = theta - numpy.asarray(diag, dtype=numpy.float64).ravel()
    small = numpy.abs(d) < floor
    d[small] = numpy.where(d[small] < 0.0, -floor, floor)
    return d


def precondition(params, r, diag, theta, f, floor):
    """t = m * r / d (the fused inference + preconditioning kernel)."""
    return forward(params, f) * numpy.asarray(r).ravel() / floored(diag, theta, floor)


def loss_and_dm(m, u, x, a):
    """Loss L(m) and dL/dm (per determinant)."""
    u, x, a = (numpy.asarray(v).ravel() for v in (u, x, a))
    w = m * u
    c = numpy.vdot(x, w)
    v = w - x * c
    s = numpy.vdot(a, v)
    q = numpy.vdot(v, v).real
    A = numpy.vdot(a, a).real
    L = 1.0 - abs(s) ** 2 / (A * q)
    ds = 2.0 * (numpy.conj(s) * numpy.conj(a) * u).real
    dq = 2.0 * (numpy.conj(v) * u).real
    dm = -(ds * q - abs(s) ** 2 * dq) / (A * q * q)
    return L, dm


def loss_and_grad(params, f, u, x, a, rounding=True):
    """Loss and d loss / d params (gradient taken at the bf16-rounded
    weights and applied to the float32 master copy; rounding=False gives the
    exact gradient of the unrounded network, for finite differences)."""
    m, (w, f, z1, h1, z2, h2) = forward(params, f, cache=True,
                                         rounding=rounding)
    L, dm = loss_and_dm(m, u, x, a)
    d3 = dm * (1.0 - (m - 1.0) ** 2)
    g = {"w3": h2.T @ d3, "b3": numpy.array([d3.sum()])}
    d2 = numpy.outer(d3, w["w3"]) * (z2 > 0.0)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(axis=0)
    d1 = (d2 @ w["W2"]) * (z1 > 0.0)
    g["W1"] = d1.T @ f
    g["b1"] = d1.sum(axis=0)
    grad = numpy.concatenate([g[name].ravel() for name, _ in SIZES])
    return L, grad


def init_params(seed=0):
    """He-initialised hidden layers, zero output layer (m = 1 at start: the
    untrained network is the plain diagonal preconditioner)."""
    rng = numpy.random.default_rng(seed)
    w = {"W1": rng.normal(0.0, (2.0 / NIN) ** 0.5, (NH, NIN)),
         "b1": numpy.zeros(NH),
         "W2": rng.normal(0.0, (2.0 / NH) ** 0.5, (NH, NH)),
         "b2": numpy.zeros(NH), "w3": numpy.zeros(NH), "b3": numpy.zeros(1)}
    return numpy.concatenate([w[n].ravel() for n, _ in SIZES]).astype(numpy.float32)


def adam(params, grad, state, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step on the float32 master copy (float64 arithmetic)."""
    m1, m2, t = state
    t += 1
    m1 = beta1 * m1 + (1 - beta1) * grad
    m2 = beta2 * m2 + (1 - beta2) * grad * grad
    mh = m1 / (1 - beta1 ** t)
    vh = m2 / (1 - beta2 ** t)
    p = params.astype(numpy.float64) - lr * mh / (numpy.sqrt(vh) + eps)
    return p.astype(numpy.float32), (m1, m2, t)
