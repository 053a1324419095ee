"""Learned surrogate of the body-frame resistance tensor of superellipsoids.

The batched BEM (:func:`andromeda_gb300.api.batch_resistance`) generates
training tensors; an MLP 5 -> 256 -> 256 -> 256 -> 21 (SiLU, BF16 tensor-core
GEMMs with FP32 accumulation, trained on the GPU by the library's own forward,
backward and Adam kernels) maps the shape parameters (b, c, e1, e2, log aspect)
of a superellipsoid with a = 1 to the 21 upper-triangle entries of its
symmetric 6x6 translation/rotation resistance tensor.  An ensemble of such
networks answers a query when it lies inside the training hull (an axis box
plus a Mahalanobis guard) and the members agree within a threshold calibrated
on held-out BEM tensors; every other query is answered by the BEM itself, and
a random audit subset is re-solved by the BEM to judge the surrogate's error.
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


def shape_scale(params):
    """[n, 6, 6] scale of the tensor entries: with the volume-equivalent radius
    r = (a b c)^(1/3) (a = 1), force-velocity entries grow as r, couplings as
    r^2, torque-rotation entries as r^3.  Dividing by it leaves O(1) targets of
    similar size for every shape, so that the network's error is a similar
    fraction of every body's tensor (the error measure is relative per body)."""
    p = np.asarray(params, dtype=np.float64)
    r = np.cbrt(p[:, 0] * p[:, 1])
    k = np.array([0, 0, 0, 1, 1, 1])
    return r[:, None, None] ** (1 + k[None, :, None] + k[None, None, :])


def tensor_to_targets(R, params=None):
    """[n, 6, 6] tensors -> [n, 21] upper triangle of the symmetric part (divided
    by shape_scale when the shapes are given)."""
    R = np.asarray(R, dtype=np.float64)
    S = 0.5 * (R + np.swapaxes(R, 1, 2))
    if params is not None:
        S = S / shape_scale(params)
    return S[:, IU[0], IU[1]].astype(np.float32)


def targets_to_tensor(y, params=None):
    y = np.asarray(y, dtype=np.float64)
    R = np.zeros((len(y), 6, 6))
    R[:, IU[0], IU[1]] = y
    R[:, IU[1], IU[0]] = y
    if params is not None:
        R = R * shape_scale(params)
    return R


def rel_err(R, Rt):
    """Max-entry relative error per body (the tensor error of the workload)."""
    R, Rt = np.asarray(R), np.asarray(Rt)
    return np.max(np.abs(R - Rt), axis=(1, 2)) / np.max(np.abs(Rt), axis=(1, 2))


def bem_tensors(params, n_elem=500, outer_level=2, outer_radius=200.0, eps=3e-8, ctx=None, solver=None):
    """Body-frame resistance tensors of superellipsoids (a = 1, b, c, e1, e2;
    no rotation) by the batched mixed-precision BEM, each body inside its own
    container sphere.  Returns (R [n, 6, 6], stats)."""
    meshes = []
    for b, c, e1, e2 in np.asarray(params, dtype=np.float64)[:, :4]:
        body = M.superellipsoid_tri(1.0, b, c, e1, e2, n_elem, inward=True)
        meshes.append(M.particle_in_sphere(body, outer_level=outer_level, outer_radius=outer_radius))
    kw = {} if solver is None else {"solver": solver}
    R, nit, istop, st = batch_resistance(meshes, eps=eps, ctx=ctx, **kw)
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
    """An ensemble of MLPs + training hull + BEM fallback.

    The members differ in their initial weights, their batch order and the
    random 85 % of the training tensors each one sees.  A query inside the training hull is answered by the
    members' mean when their spread (max-entry distance of the members from the
    mean, relative to the mean's largest entry) is at most ``tau``; ``tau`` is
    calibrated on held-out BEM tensors (:meth:`calibrate`) so that every
    accepted held-out answer is within the target error.  Every other query --
    outside the hull or with a larger spread -- is answered by the BEM."""

    def __init__(self, device=0, seed=1, bem_kwargs=None, members=4):
        self.nets = [MLP(device=device, seed=seed + 7919 * k) for k in range(max(1, members))]
        self.net = self.nets[0]
        self.hull = Hull()
        self.bem_kwargs = dict(bem_kwargs or {})
        self.tau = np.inf

    def close(self):
        for n in self.nets:
            n.close()

    def fit(self, params, R, epochs=400, batch=512, lr=1e-3, lr_final=1e-5, seed=0, subsample=0.85):
        """Train every member on BEM tensors R of shapes `params` -- each on its
        own random `subsample` of them (bagging: the members differ most where
        the data are thin, which is where their spread should flag a query);
        the learning rate decays geometrically from lr to lr_final over four
        stages of the epochs.  Returns (loss history of the first member,
        summed stats)."""
        X_all = features(params)
        Y_all = tensor_to_targets(R, params)
        self.hull.fit(X_all)
        X, Y = X_all, Y_all
        xm, xs = X.mean(axis=0), X.std(axis=0) + 1e-6
        ym = Y.mean(axis=0)
        ys = Y.std(axis=0)
        ys = np.maximum(ys, 1e-3 * np.max(ys))  # near-constant entries (symmetric shapes) keep a sane scale
        hist0, total = None, {"device_ms": 0.0, "launches": 0, "adam_steps": 0}
        stages = 4
        for mi, net in enumerate(self.nets):
            net.set_normalization(xm, xs, ym, ys)
            if subsample < 1.0 and len(self.nets) > 1:
                pick = np.random.default_rng(seed + 7919 * mi).permutation(len(X_all))[:int(subsample * len(X_all))]
                X, Y = X_all[np.sort(pick)], Y_all[np.sort(pick)]
            hist = []
            for k in range(stages):
                e = epochs // stages + (1 if k < epochs % stages else 0)
                lr_k = lr * (lr_final / lr) ** (k / max(stages - 1, 1))
                h, st = net.train(X, Y, e, batch=batch, lr=lr_k, seed=seed + 1009 * mi + k)
                hist.extend(h.tolist())
                total["device_ms"] += st["device_ms"]
                total["launches"] += st["launches"]
                total["adam_steps"] += st["adam_steps"]
            if hist0 is None:
                hist0 = np.array(hist)
        return hist0, total

    def ensemble(self, X):
        """Members' mean targets [n, 21], their spread [n] and the summed kernel
        time (ms) for features X."""
        ys, ms = [], 0.0
        for net in self.nets:
            y, t = net.predict(X)
            ys.append(y.astype(np.float64))
            ms += t
        Ys = np.stack(ys)
        mean = Ys.mean(axis=0)
        scale = np.max(np.abs(mean), axis=1)
        spread = np.max(np.abs(Ys - mean[None]), axis=(0, 2)) / np.maximum(scale, 1e-300)
        return mean, spread, ms

    def calibrate(self, params, R, target=1e-3, margin=0.8):
        """Largest spread threshold tau under which every held-out answer
        (params, BEM tensors R) inside the hull is within margin * target of
        the BEM.  Returns a summary of the held-out set."""
        X = features(params)
        inside = self.hull.contains(X)
        mean, spread, _ = self.ensemble(X[inside])
        err = rel_err(targets_to_tensor(mean, np.asarray(params)[inside]), np.asarray(R)[inside])
        order = np.argsort(spread)
        ok = np.cumsum(err[order] > margin * target) == 0
        nacc = int(np.sum(ok))  # a prefix of the spread-sorted held-out answers
        self.tau = float(spread[order][nacc - 1]) if nacc > 0 else 0.0
        return {"n": int(len(X)), "in_hull": int(inside.sum()), "accepted": nacc, "tau": self.tau,
                "err_median": float(np.median(err)) if len(err) else None,
                "err_max_accepted": float(np.max(err[order][:nacc])) if nacc else None}

    def predict(self, params, bem=True):
        """Tensors for `params`: the ensemble where the query is inside the hull
        and the members agree within tau, the BEM elsewhere (bem=False leaves
        NaN there).  Returns (R, accepted mask, info)."""
        X = features(params)
        inside = self.hull.contains(X)
        R = np.full((len(X), 6, 6), np.nan)
        acc = np.zeros(len(X), bool)
        ms = 0.0
        if inside.any():
            mean, spread, ms = self.ensemble(X[inside])
            ok = spread <= self.tau
            idx = np.where(inside)[0]
            acc[idx[ok]] = True
            R[idx[ok]] = targets_to_tensor(mean[ok], np.asarray(params)[idx[ok]])
        info = {"mlp_device_ms": ms, "n_mlp": int(acc.sum()), "n_bem": int((~acc).sum()),
                "n_outside_hull": int((~inside).sum()), "n_spread_rejected": int((inside & ~acc).sum())}
        if bem and (~acc).any():
            Rb, st = bem_tensors(np.asarray(params)[~acc], **self.bem_kwargs)
            R[~acc] = Rb
            info["bem_ms"] = st["device_ms"]
        return R, acc, info

    def audit(self, params, frac=0.01, seed=0):
        """BEM re-solve of a random fraction of the queries: max-entry relative
        errors of the accepted surrogate answers among them, and which were
        accepted."""
        rng = np.random.default_rng(seed)
        n = len(params)
        k = max(1, int(round(frac * n)))
        idx = np.sort(rng.choice(n, size=k, replace=False))
        sub = np.asarray(params)[idx]
        R, acc, _ = self.predict(sub, bem=False)
        Rb, st = bem_tensors(sub, **self.bem_kwargs)
        err = rel_err(R[acc], Rb[acc]) if acc.any() else np.zeros(0)
        return err, idx, acc, st
