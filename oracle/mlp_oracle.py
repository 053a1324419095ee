"""FP64 CPU oracle of the MLP surrogate -- TEST INFRASTRUCTURE ONLY.

Forward and backward of the network nin -> nh -> nh -> nh -> nout with SiLU
and the mean squared error of normalised outputs, in numpy float64, with the
parameter layout of the C ABI (W1 [nh][nin], b1, W2 [nh][nh], b2, W3, b3,
W4 [nout][nh], b4).  The GPU gradients of agb_mlp_gradient are checked
against it.  There is no reference counterpart: the surrogate is new.
"""
import numpy as np


def unpack(p, nin=5, nh=256, nout=21):
    p = np.asarray(p, dtype=np.float64)
    sizes = [(nh, nin), (nh,), (nh, nh), (nh,), (nh, nh), (nh,), (nout, nh), (nout,)]
    out, o = [], 0
    for s in sizes:
        k = int(np.prod(s))
        out.append(p[o:o + k].reshape(s))
        o += k
    assert o == len(p)
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, Xn, nin=5, nh=256, nout=21):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p, nin, nh, nout)
    Z1 = Xn @ W1.T + b1
    H1 = silu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = silu(Z2)
    Z3 = H2 @ W3.T + b3
    H3 = silu(Z3)
    Y = H3 @ W4.T + b4
    return Y, (Xn, Z1, H1, Z2, H2, Z3, H3)


def loss_and_grad(p, X, T, xm, xs, ym, ys, nin=5, nh=256, nout=21):
    """Mean squared error of the normalised outputs and its gradient."""
    Xn = (np.asarray(X, np.float64) - xm) / xs
    Tn = (np.asarray(T, np.float64) - ym) / ys
    Y, (Xn, Z1, H1, Z2, H2, Z3, H3) = forward(p, Xn, nin, nh, nout)
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p, nin, nh, nout)
    n = len(X)
    d = Y - Tn
    loss = np.mean(d * d)
    dY = 2.0 * d / (n * nout)
    gW4 = dY.T @ H3
    gb4 = dY.sum(axis=0)
    dZ3 = (dY @ W4) * dsilu(Z3)
    gW3 = dZ3.T @ H2
    gb3 = dZ3.sum(axis=0)
    dZ2 = (dZ3 @ W3) * dsilu(Z2)
    gW2 = dZ2.T @ H1
    gb2 = dZ2.sum(axis=0)
    dZ1 = (dZ2 @ W2) * dsilu(Z1)
    gW1 = dZ1.T @ Xn
    gb1 = dZ1.sum(axis=0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4)])
    return loss, g
