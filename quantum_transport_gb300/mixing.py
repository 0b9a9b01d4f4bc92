"""Learned SCBA mixing: a network proposes the next self-energy iterate.

The reference iterates Sigma <- Sigma + alpha (F(Sigma) - Sigma) with a fixed
alpha (src/gw_mod.f90:747-749), F being one GW evaluation (G by RGF, P, W,
Sigma; ``GwSystem.step``).  Here every accepted iterate enters a short history
of (Sigma_j, R_j = F(Sigma_j) - Sigma_j).  Pulay's DIIS combination
(coefficients c, sum c = 1, minimising ||sum c_j R_j||) gives

    Sigma_bar = sum c_j Sigma_j,      R_bar = sum c_j R_j,

and a Pulay step moves to Sigma_bar + alpha R_bar.  The network instead chooses
the step length per orbital o (row i of slab l):

    Sigma_new = Sigma_bar + a_ij R_bar,      a_ij = (a_i + a_j)/2,

applied to Sigma^R, Sigma^< and Sigma^>.  It reads, per orbital, the Chebyshev
coefficients of the diagonal series Im R^<_ii(E), Im R^>_ii(E) of R_bar and of
the last two residuals, plus the global residual and the orbital's DIIS
reduction |R_bar| / |R_k|.  At a fixed point every R_j = 0, so no proposal can
move the fixed point.  A proposal is kept only if the residual F evaluates for
it falls below ACCEPT_RATIO times the last accepted one; otherwise it is
discarded, the Pulay step is taken instead, and so are the next COOLDOWN steps.

Training data come from the method itself: Pulay runs (the loop without the
network) on seeded disorder realisations give iterate histories and their
converged fixed point Sigma*.  For each iterate and orbital the target a* is
the least-squares step along R_bar towards Sigma* over both diagonal series.
Further rounds add the learned loop's own iterates with the same targets.  The
network is trained on the GPU by the library's own kernels (``mlp.Mlp``).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import time

import numpy as np

from ._lib import check
from .mlp import Mlp

NCOEF = 64
NHIST = 3            # series per feature row: R_bar, R_k, R_{k-1}
N_IN = 2 * NHIST * NCOEF + 2
N_OUT = 1
ALPHA_MAX = 4.0      # largest step along R_bar
ACCEPT_RATIO = 0.8   # a learned proposal is kept only if it cuts the residual by >= 20 %
COOLDOWN = 2         # Pulay steps after a rejected proposal before the network is asked again


def chebyshev_projector(nE, ncoef=NCOEF):
    """Qt (nE, ncoef): least-squares Chebyshev coefficients c = Qt^T s of a series
    s sampled on a uniform grid mapped to [-1, 1]."""
    x = np.linspace(-1.0, 1.0, nE)
    V = np.polynomial.chebyshev.chebvander(x, ncoef - 1)
    return np.ascontiguousarray(np.linalg.pinv(V).T)


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _plist(ts):
    arr = (C.c_void_p * len(ts))(*[t.data_ptr() for t in ts])
    return C.cast(arr, C.POINTER(C.c_void_p)), arr


class MixOps:
    """Self-energy arithmetic on the device through the mixing kernels."""

    def __init__(self, system):
        self.sys = system
        self.ctx = system.ctx
        self.lib = system.ctx._lib
        self.count = system.nE * system.nx * system.nm * system.nm

    def combine(self, coef, X, R, alpha, out):
        px, kx = _plist(X)
        pr, kr = _plist(R)
        c = np.ascontiguousarray(coef, dtype=np.float64)
        check(self.lib.qt_mix_combine(self.ctx.handle, self.count, len(X),
                                      c.ctypes.data_as(C.c_void_p), px, pr, float(alpha),
                                      _vp(out), 0))
        return out

    def diff(self, N, S, out):
        """out = N - S"""
        return self.combine([1.0], [N], [S], -1.0, out)

    def gram(self, XL, XG):
        k = len(XL)
        G = np.zeros((k, k))
        pl, kl = _plist(XL)
        pg, kg = _plist(XG)
        check(self.lib.qt_mix_gram(self.ctx.handle, self.count, k, pl, pg,
                                   G.ctypes.data_as(C.c_void_p)))
        return G

    def residual(self, R, N):
        """||R^<, R^>|| / ||N^<, N^>|| (the SCBA stopping measure)"""
        G = self.gram([R[1], N[1]], [R[2], N[2]])
        return float(np.sqrt(G[0, 0]) / max(np.sqrt(G[1, 1]), 1e-300))

    def diag(self, XL, XG, out):
        s = self.sys
        check(self.lib.qt_mix_diag(self.ctx.handle, s.nE, s.nx, s.nm, _vp(XL), _vp(XG),
                                   _vp(out), 0))
        return out


def pulay_coefficients(G):
    """DIIS: minimise || sum c_i R_i || with sum c_i = 1 (G: residual Gram matrix)."""
    k = G.shape[0]
    scale = max(np.abs(np.diag(G)).max(), 1e-300)
    A = np.zeros((k + 1, k + 1))
    A[:k, :k] = G / scale
    A[k, :k] = A[:k, k] = 1.0
    b = np.zeros(k + 1)
    b[k] = 1.0
    return np.linalg.lstsq(A, b, rcond=None)[0][:k]


@dataclasses.dataclass
class ScbaResult:
    sigma: tuple          # (Sigma^R, Sigma^<, Sigma^>) device tensors
    residuals: list       # residual of every evaluation of F
    evaluations: int      # GW evaluations (iterations), rejected proposals included
    seconds: float
    accepted: int = 0     # learned proposals kept
    rejected: int = 0     # learned proposals discarded (Pulay step taken instead)
    pulay: int = 0        # Pulay steps
    plain: int = 0        # linear-mixing steps
    kinds: list = dataclasses.field(default_factory=list)  # step that produced each evaluation


class Recorder:
    """Collects network inputs and the diagonal series of (Sigma_bar, R_bar) of one run,
    from which training targets follow once the fixed point is known."""

    def __init__(self):
        self.feats, self.s, self.r = [], [], []

    def add(self, feats, s_diag, r_diag):
        self.feats.append(feats)
        self.s.append(s_diag)
        self.r.append(r_diag)

    def targets(self, s_star):
        """(X, T): network inputs and the step a* along R_bar that brings each orbital's
        diagonal closest to the fixed point's (least squares over both series)."""
        if not self.feats:
            return np.zeros((0, N_IN), np.float32), np.zeros((0, N_OUT), np.float32)
        X, T = [], []
        for f, s, r in zip(self.feats, self.s, self.r):
            u = (s_star - s).reshape(-1, s.shape[-1])  # [2 nE][norb]
            r = r.reshape(u.shape)
            a = (r * u).sum(0) / ((r * r).sum(0) + 1e-300)
            T.append(np.clip(a, 0.0, ALPHA_MAX)[:, None])
            X.append(f)
        return np.concatenate(X).astype(np.float32), np.concatenate(T).astype(np.float32)


class LearnedMixer:
    """The network and the Chebyshev projector for one energy grid."""

    def __init__(self, ctx, nE, *, width=512, depth=4, max_batch=1 << 16, seed=0, params=None):
        import torch
        self.ctx = ctx
        self.nE = nE
        self.Qt = torch.from_numpy(chebyshev_projector(nE)).cuda()
        self.net = Mlp(ctx, N_IN, width, depth, N_OUT, max_batch, params=params, seed=seed)

    def features(self, ring, log_residual, out):
        norb = ring.shape[-1]
        check(self.ctx._lib.qt_mix_features(self.ctx.handle, self.nE, norb, NHIST, _vp(ring),
                                            _vp(self.Qt), float(log_residual), _vp(out), 0))
        return out


def _diis(ops, hist):
    """Sigma_bar, R_bar (three tensors each) of the DIIS combination of ``hist``."""
    import torch
    G = ops.gram([h[1][1] for h in hist], [h[1][2] for h in hist])
    c = pulay_coefficients(G)
    zero = [h[1][0] for h in hist]  # any tensors: alpha = 0 ignores them
    Sb = tuple(ops.combine(c, [h[0][q] for h in hist], zero, 0.0, torch.empty_like(hist[-1][0][q]))
               for q in range(3))
    Rb = tuple(ops.combine(c, [h[1][q] for h in hist], zero, 0.0, torch.empty_like(hist[-1][1][q]))
               for q in range(3))
    return Sb, Rb


def _step(system, Sb, Rb, a=None, alpha=0.3):
    """Sigma_bar + alpha R_bar, or Sigma_bar + a_ij R_bar with per-orbital a (device [norb][1])."""
    import torch
    ops = MixOps(system)
    if a is None:
        return tuple(ops.combine([1.0], [Sb[q]], [Rb[q]], alpha, torch.empty_like(Sb[q]))
                     for q in range(3))
    out = []
    for q in range(3):
        o = torch.empty_like(Sb[q])
        check(system.ctx._lib.qt_mix_apply(
            system.ctx.handle, system.nE, system.nx, system.nm, _vp(a), 1, ALPHA_MAX, 0.0, 0.0,
            _vp(Sb[q]), _vp(Rb[q]), None, _vp(o), 0))
        out.append(o)
    return tuple(out)


def run_scba(system, *, method="learned", mixer=None, alpha=0.3, tol=1e-8, max_iter=60,
             pulay_depth=3, recorder=None):
    """SCBA to ||R|| / ||F(Sigma)|| <= tol with plain, Pulay or learned mixing.

    ``method``: "plain" (the reference's linear mixing), "pulay" (DIIS over the
    last ``pulay_depth`` accepted iterates, step alpha along R_bar) or "learned"
    (network step lengths along R_bar, Pulay fallback).  Returns a ``ScbaResult``;
    the converged self-energy is Sigma + alpha R of the last evaluation, as in the
    plain loop.
    """
    import torch
    if method not in ("plain", "pulay", "learned"):
        raise ValueError("method is plain, pulay or learned")
    if method == "learned" and mixer is None:
        raise ValueError("learned mixing needs a LearnedMixer")
    ops = MixOps(system)
    norb = system.nx * system.nm
    S = (system.zeros(), system.zeros(), system.zeros())
    hist, rdiag = [], []  # accepted (Sigma, R) and their residual diagonal series
    ring = torch.zeros((NHIST, 2, system.nE, norb), dtype=torch.float64, device="cuda")
    feats = torch.empty((norb, N_IN), dtype=torch.float32, device="cuda")
    a = torch.empty((norb, N_OUT), dtype=torch.float32, device="cuda")
    res = ScbaResult(sigma=None, residuals=[], evaluations=0, seconds=0.0)
    r_acc, last, final = np.inf, None, None
    cool = 0  # Pulay steps left before the network is asked again
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max_iter):
        N = system.step(S[0], S[1])
        R = tuple(ops.diff(N[q], S[q], torch.empty_like(S[q])) for q in range(3))
        r = ops.residual(R, N)
        res.residuals.append(r)
        res.kinds.append(last or "start")
        if r <= tol:
            final = tuple(ops.combine([1.0], [S[q]], [R[q]], alpha, torch.empty_like(S[q]))
                          for q in range(3))
            if last == "learned":
                res.accepted += 1
            break
        if last == "learned" and r >= ACCEPT_RATIO * r_acc:
            res.rejected += 1
            S = _step(system, *_diis(ops, hist[-pulay_depth:]), alpha=alpha)
            res.pulay += 1
            last = "pulay"
            cool = COOLDOWN
            continue
        if last == "learned":
            res.accepted += 1
        hist = (hist + [(S, R)])[-pulay_depth:]
        rd = torch.empty((2, system.nE, norb), dtype=torch.float64, device="cuda")
        rdiag = (rdiag + [ops.diag(R[1], R[2], rd)])[-2:]
        r_acc = r
        if method == "plain" or len(hist) < 2:
            S = tuple(ops.combine([1.0], [S[q]], [R[q]], alpha, torch.empty_like(S[q]))
                      for q in range(3))
            res.plain += 1
            last = "plain"
            continue
        Sb, Rb = _diis(ops, hist)
        use_net = method == "learned" and cool == 0
        if use_net or recorder is not None:
            ops.diag(Rb[1], Rb[2], ring[0])
            ring[1].copy_(rdiag[-1])
            ring[2].copy_(rdiag[-2])
            (mixer.features if mixer is not None else _features_only(system))(
                ring, np.log10(max(r, 1e-300)), feats)
        if recorder is not None:
            sd = ops.diag(Sb[1], Sb[2], torch.empty_like(ring[0]))
            recorder.add(feats.cpu().numpy(), sd.cpu().numpy(), ring[0].cpu().numpy())
        if use_net:
            mixer.net.infer(feats, out=a)
            S = _step(system, Sb, Rb, a=a)
            last = "learned"
        else:
            cool = max(cool - 1, 0)
            S = _step(system, Sb, Rb, alpha=alpha)
            res.pulay += 1
            last = "pulay"
    torch.cuda.synchronize()
    res.seconds = time.perf_counter() - t0
    res.sigma = final if final is not None else S
    res.evaluations = len(res.residuals)
    return res


_FEATURE_CACHE = {}


def _features_only(system):
    """Feature extraction without a network (recording plain runs)."""
    import torch
    key = (id(system.ctx), system.nE)
    if key not in _FEATURE_CACHE:
        Qt = torch.from_numpy(chebyshev_projector(system.nE)).cuda()

        def f(ring, log_residual, out, Qt=Qt, ctx=system.ctx, nE=system.nE):
            check(ctx._lib.qt_mix_features(ctx.handle, nE, ring.shape[-1], NHIST, _vp(ring),
                                           _vp(Qt), float(log_residual), _vp(out), 0))
            return out
        _FEATURE_CACHE[key] = f
    return _FEATURE_CACHE[key]


def fixed_point_diag(system, result):
    """Diagonal series [2][nE][norb] of a converged result's Sigma^<, Sigma^>."""
    import torch
    ops = MixOps(system)
    out = torch.empty((2, system.nE, system.nx * system.nm), dtype=torch.float64, device="cuda")
    return ops.diag(result.sigma[1], result.sigma[2], out).cpu().numpy()


def collect(systems, *, mixer=None, alpha=0.3, tol=1e-8, max_iter=200, fixed_points=None):
    """Training pairs from SCBA runs on ``systems`` (a list of GwSystem).

    Without ``mixer``: Pulay runs (the loop without the network), whose converged
    result is the fixed point.  With ``mixer``: learned runs, targets taken against
    ``fixed_points`` (one diagonal series per system, from the Pulay runs).
    Returns (X, T, fixed_points, results).
    """
    Xs, Ts, fps, results = [], [], [], []
    for i, s in enumerate(systems):
        rec = Recorder()
        r = run_scba(s, method="pulay" if mixer is None else "learned", mixer=mixer,
                     alpha=alpha, tol=tol, max_iter=max_iter, recorder=rec)
        fp = fixed_point_diag(s, r) if mixer is None else fixed_points[i]
        X, T = rec.targets(fp)
        Xs.append(X)
        Ts.append(T)
        fps.append(fp)
        results.append(r)
    return np.concatenate(Xs), np.concatenate(Ts), fps, results


def train(mixer, X, T, *, steps=1500, batch=4096, lr=1e-3, weight_decay=1e-4, seed=0,
          log_every=0):
    """AdamW on the GPU with the library's kernels; returns the loss trace (host).

    A fresh network first gets its output layer set to predict the targets' mean (bias =
    mean, weights scaled by 0.1), so that training fits the per-orbital variation.
    """
    import torch
    if not getattr(mixer, "trained", False):
        p = mixer.net.params()
        d = mixer.net.dims  # (n_in, width, depth, n_out)
        wo = mixer.net.nparams - d[3] - d[1] * d[3]
        p[wo:wo + d[1] * d[3]] *= 0.1
        p[wo + d[1] * d[3]:] = np.asarray(T, np.float64).mean(axis=0)
        mixer.net.set_params(p)
        mixer.trained = True
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    Td = torch.from_numpy(np.ascontiguousarray(T, np.float32)).cuda()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n = Xd.shape[0]
    b = min(batch, n, mixer.net.max_batch)
    losses = []
    for step in range(steps):
        idx = torch.randint(0, n, (b,), device="cuda", generator=g)
        want = log_every and (step % log_every == 0 or step == steps - 1)
        loss = mixer.net.train_step(Xd[idx].contiguous(), Td[idx].contiguous(), lr=lr,
                                    weight_decay=weight_decay, want_loss=bool(want))
        if want:
            losses.append((step, loss))
    return losses
