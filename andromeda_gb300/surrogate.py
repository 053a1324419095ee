"""Learned surrogate of the body-frame resistance tensor of superellipsoids.

The batched BEM (:func:`andromeda_gb300.api.batch_resistance`) generates
training tensors; an MLP 5 -> 256 -> 256 -> 256 -> 21 (SiLU, BF16 tensor-core
GEMMs with FP32 accumulation, trained on the GPU by the library's own forward,
backward and Adam kernels) maps the shape parameters (b, c, e1, e2, log aspect)
of a superellipsoid with a = 1 to the 21 upper-triangle entries of its
symmetric 6x6 translation/rotation resistance tensor.  Queries outside the
training hull (an axis box plus a Mahalanobis guard) are answered by the BEM
itself, and a random audit subset is re-solved by the BEM to judge the
surrogate's error.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import mesh as M
from ._lib import AgbError, load
from .api import batch_resistance

IU = np.triu_indices(6)  # the 21 independent entries, row-major upper triangle


def features(params):
    """(b, c, e1, e2) rows -> (b, c, e1, e2, log aspect) with a = 1 >= b, c."""
    p = np.asarray(params, dtype=np.float64)[:, :4]
    aspect = 1.0 / np.minimum(p[:, 0], p[:, 1])
    return np.column_stack([p, np.log(aspect)]).astype(np.float32)


def tensor_to_targets(R):
    """[n, 6, 6] tensors -> [n, 21] upper triangle of the symmetric part."""
    R = np.asarray(R, dtype=np.float64)
    S = 0.5 * (R + np.swapaxes(R, 1, 2))
    return S[:, IU[0], IU[1]].astype(np.float32)


def targets_to_tensor(y):
    y = np.asarray(y, dtype=np.float64)
    R = np.zeros((len(y), 6, 6))
    R[:, IU[0], IU[1]] = y
    R[:, IU[1], IU[0]] = y
    return R


def rel_err(R, Rt):
    """Max-entry relative error per body (the tensor error of the workload)."""
    R, Rt = np.asarray(R), np.asarray(Rt)
    return np.max(np.abs(R - Rt), axis=(1, 2)) / np.max(np.abs(Rt), axis=(1, 2))


def bem_tensors(params, n_elem=400, outer_level=1, outer_radius=20.0, eps=3e-8, ctx=None):
    """Body-frame resistance tensors of superellipsoids (a = 1, b, c, e1, e2;
    no rotation) by the batched mixed-precision BEM, each body inside its own
    container sphere.  Returns (R [n, 6, 6], stats)."""
    meshes = []
    for b, c, e1, e2 in np.asarray(params, dtype=np.float64)[:, :4]:
        body = M.superellipsoid_tri(1.0, b, c, e1, e2, n_elem, inward=True)
        meshes.append(M.particle_in_sphere(body, outer_level=outer_level, outer_radius=outer_radius))
    R, nit, istop, st = batch_resistance(meshes, eps=eps, ctx=ctx)
    return R, st


def sample_params(n, seed):
    """Shape parameters of the many-body workload: b, c ~ U(0.2, 1), e1, e2 ~ U(0.3, 1.8)."""
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(0.2, 1.0, (n, 2)), rng.uniform(0.3, 1.8, (n, 2))])


class Hull:
    """Training hull: the axis box of the training features plus a Mahalanobis
    guard at the largest training distance."""

    def fit(self, X):
        X = np.asarray(X, dtype=np.float64)
        self.lo, self.hi = X.min(axis=0), X.max(axis=0)
        self.mu = X.mean(axis=0)
        self.icov = np.linalg.inv(np.cov(X.T) + 1e-12 * np.eye(X.shape[1]))
        self.d2max = float(np.max(self._d2(X)))
        return self

    def _d2(self, X):
        d = np.asarray(X, dtype=np.float64) - self.mu
        return np.einsum("ij,jk,ik->i", d, self.icov, d)

    def contains(self, X):
        X = np.asarray(X, dtype=np.float64)
        box = np.all((X >= self.lo) & (X <= self.hi), axis=1)
        return box & (self._d2(X) <= self.d2max)


class MLP:
    """The network on the GPU (agb_mlp_* of the C ABI)."""

    def __init__(self, device=0, nin=5, nhidden=256, nout=21, seed=1):
        self._L = load()
        h = C.c_void_p()
        rc = self._L.agb_mlp_create(C.byref(h), int(device), nin, nhidden, nout, int(seed))
        if rc:
            raise AgbError(f"agb_mlp_create failed ({rc}): {self._L.agb_last_error(None).decode()}")
        self.h, self.nin, self.nout = h, nin, nout
        n = C.c_longlong()
        self._ck(self._L.agb_mlp_num_params(self.h, C.byref(n)))
        self.nparams = n.value

    def _ck(self, rc):
        if rc:
            raise AgbError(f"andromeda_gb300 error {rc}: {self._L.agb_last_error(None).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self._L.agb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(self.nparams, np.float32)
        self._ck(self._L.agb_mlp_get_params(self.h, p))
        return p

    def set_params(self, p):
        self._ck(self._L.agb_mlp_set_params(self.h, np.ascontiguousarray(p, dtype=np.float32)))

    def set_normalization(self, xm, xs, ym, ys):
        f = lambda v: np.ascontiguousarray(v, dtype=np.float32)  # noqa: E731
        self._ck(self._L.agb_mlp_set_normalization(self.h, f(xm), f(xs), f(ym), f(ys)))

    def gradient(self, X, Y, split=False):
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_double()
        self._ck(self._L.agb_mlp_gradient(self.h, len(X), np.ascontiguousarray(X, dtype=np.float32),
                                          np.ascontiguousarray(Y, dtype=np.float32), int(bool(split)), g,
                                          C.byref(loss)))
        return g, loss.value

    def train(self, X, Y, epochs, batch=512, lr=1e-3, seed=0):
        hist = np.zeros(epochs)
        st = np.zeros(3)
        self._ck(self._L.agb_mlp_train(self.h, len(X), np.ascontiguousarray(X, dtype=np.float32),
                                       np.ascontiguousarray(Y, dtype=np.float32), int(epochs), int(batch), float(lr),
                                       int(seed), hist, st))
        return hist, {"device_ms": st[0], "launches": int(st[1]), "adam_steps": int(st[2])}

    def predict(self, X, split=True, fused=True):
        """Outputs for X (physical units) and the kernel time in ms.  split:
        split-BF16 products (FP32-level accuracy); fused: one kernel for all
        layers (split only), else the layer-by-layer GEMMs."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((len(X), self.nout), np.float32)
        ms = C.c_double()
        mode = (1 if fused else 2) if split else 0
        self._ck(self._L.agb_mlp_predict(self.h, len(X), X, Y, mode, C.byref(ms)))
        return Y, ms.value


class Surrogate:
    """MLP + training hull + BEM fallback."""

    def __init__(self, device=0, seed=1, bem_kwargs=None):
        self.net = MLP(device=device, seed=seed)
        self.hull = Hull()
        self.bem_kwargs = dict(bem_kwargs or {})

    def fit(self, params, R, epochs=400, batch=512, lr=1e-3, lr_final=1e-5, seed=0):
        """Train on BEM tensors R of shapes `params`; the learning rate decays
        geometrically from lr to lr_final over four stages of the epochs."""
        X = features(params)
        Y = tensor_to_targets(R)
        self.hull.fit(X)
        xm, xs = X.mean(axis=0), X.std(axis=0) + 1e-6
        ym = Y.mean(axis=0)
        ys = Y.std(axis=0)
        ys = np.maximum(ys, 1e-3 * np.max(ys))  # near-constant entries (symmetric shapes) keep a sane scale
        self.net.set_normalization(xm, xs, ym, ys)
        hist, total = [], {"device_ms": 0.0, "launches": 0, "adam_steps": 0}
        stages = 4
        for k in range(stages):
            e = epochs // stages + (1 if k < epochs % stages else 0)
            lr_k = lr * (lr_final / lr) ** (k / max(stages - 1, 1))
            h, st = self.net.train(X, Y, e, batch=batch, lr=lr_k, seed=seed + k)
            hist.extend(h.tolist())
            total["device_ms"] += st["device_ms"]
            total["launches"] += st["launches"]
            total["adam_steps"] = st["adam_steps"]
        return np.array(hist), total

    def predict(self, params, bem=True):
        """Tensors for `params`: the MLP inside the hull, the BEM outside
        (bem=False leaves NaN there).  Returns (R, inside mask, info)."""
        X = features(params)
        inside = self.hull.contains(X)
        R = np.full((len(X), 6, 6), np.nan)
        Y, ms = self.net.predict(X[inside])
        R[inside] = targets_to_tensor(Y)
        info = {"mlp_device_ms": ms, "n_mlp": int(inside.sum()), "n_bem": int((~inside).sum())}
        if bem and (~inside).any():
            Rb, st = bem_tensors(np.asarray(params)[~inside], **self.bem_kwargs)
            R[~inside] = Rb
            info["bem_ms"] = st["device_ms"]
        return R, inside, info

    def audit(self, params, frac=0.01, seed=0):
        """BEM re-solve of a random fraction of the queries: max-entry relative
        errors of the surrogate on them."""
        rng = np.random.default_rng(seed)
        n = len(params)
        k = max(1, int(round(frac * n)))
        idx = np.sort(rng.choice(n, size=k, replace=False))
        sub = np.asarray(params)[idx]
        R, inside, _ = self.predict(sub, bem=False)
        Rb, st = bem_tensors(sub, **self.bem_kwargs)
        err = rel_err(R[inside], Rb[inside]) if inside.any() else np.zeros(0)
        return err, idx, inside, st
