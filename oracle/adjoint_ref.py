"""FP64 reference of the differentiable float enfuse (the model enb_fuse_grad
differentiates), written with torch float64 operators so that autograd and
central finite differences give the reference gradients.

TEST INFRASTRUCTURE ONLY: the checker of the CUDA adjoint.  Only tests/ may
import it.

The model is enfuseMain's float path (src/enfuse.h:1217-1617) on opaque RGB
images, with continuous masks:
  gray   (r + g + b) / 3                               (src/mga.h:188-193)
  y      gray / range
  w_k    W_exp f((y - opt) / width') + W_con sigma + W_sat s
         f the built-in weight functions with width' the width rescaled to
         the Gaussian's FWHM (src/exposure_weight.h:44-128); sigma the sample
         standard deviation of gray in the contrast window, 0 on the border
         strip (src/enfuse.h:75-219); s the HSL saturation with max 1.0
         (src/enfuse.h:733-780)
  m_k    w_k exp(a_k) / sum_j w_j exp(a_j)             (src/enfuse.h:1526-1535, unquantised)
  pyramids of the log-mapped images and of the masks with the normalised
  5-tap reduce of opaque images and the (1,6,1)/(4,4) expand with its
  per-position divisors (src/pyramid.h:166-573, 875-1457), merge
  R[l] = sum_k LP_k[l] M_k[l] (src/enfuse.h:601-620, 1576-1588), collapse
  (src/pyramid.h:1758-1784), out = v >= 1 ? expm1(v - 1) : 1 - 1/v
  (src/fixmath.h:320-329); loss = mean((out - target)^2).
Both 1-D operators are separable, so each level step is A_h X A_w^T with
banded operator matrices, applied as sparse products (torch.sparse.mm, which
autograd differentiates in the dense factor), so that the model also runs at
2048x2048 with 8 exposures on a GPU in float64.
"""
from __future__ import annotations

import math
from typing import Sequence

import numpy as np
import torch

W5 = (1.0, 4.0, 6.0, 4.0, 1.0)
FWHM = {"gaussian": 2.3548200450309493820231386529193992755, "lorentzian": 2.8284271247461900976033774484193961571,
        "halfsine": 2.0943951023931954923084289221863352561, "fullsine": 3.14159265358979323846,
        "bisquare": 1.6817928305074290860622509524664297901}


def num_levels(w: int, h: int) -> int:
    """roiBounds' automatic level count (src/bounds.h:121-133)."""
    short = min(w, h)
    levels = 1
    while levels <= 29 and short > 8:
        short = (short + 1) >> 1
        levels += 1
    return levels


def reduce_matrix(n: int, device=None) -> torch.Tensor:
    """(ceil(n/2), n): the normalised 5-tap reduce of an opaque row."""
    m = (n + 1) >> 1
    A = torch.zeros(m, n, dtype=torch.float64)
    for I in range(m):
        taps = [(2 * I + t, W5[t + 2]) for t in range(-2, 3) if 0 <= 2 * I + t < n]
        den = sum(w for _, w in taps)
        for x, w in taps:
            A[I, x] = w / den
    return A.to(device) if device is not None else A


def expand_matrix(nf: int, nc: int, device=None) -> torch.Tensor:
    """(nf, nc): the expand of a coarse row into nf fine samples (no wrap)."""
    E = torch.zeros(nf, nc, dtype=torch.float64)
    for X in range(nf):
        i = X >> 1
        if X % 2 == 0:
            w = [1.0 if i > 0 else 0.0, 6.0, 1.0 if i + 1 < nc else 0.0]
        else:
            w = [0.0, 4.0, 4.0 if i + 1 < nc else 0.0]
        den = sum(w)
        for a in range(3):
            if w[a]:
                E[X, i + a - 1] += w[a] / den
    return E.to(device) if device is not None else E


def _rows(A: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """A @ X along the second-to-last axis: A (m, n) sparse, X (..., n, w)."""
    *lead, n, w = X.shape
    Y = torch.sparse.mm(A, X.reshape(-1, n, w).permute(1, 0, 2).reshape(n, -1))
    return Y.reshape(A.shape[0], -1, w).permute(1, 0, 2).reshape(*lead, A.shape[0], w)


def _cols(X: torch.Tensor, A: torch.Tensor) -> torch.Tensor:
    """X @ A^T along the last axis: A (m, n) sparse, X (..., h, n)."""
    *lead, h, n = X.shape
    Y = torch.sparse.mm(A, X.reshape(-1, n).T)
    return Y.T.reshape(*lead, h, A.shape[0])


def separable(Ah: torch.Tensor, X: torch.Tensor, Aw: torch.Tensor) -> torch.Tensor:
    """Ah X Aw^T on the last two axes of X with sparse operators."""
    return _cols(_rows(Ah, X), Aw)


def exposure_f(z: torch.Tensor, fn: str) -> torch.Tensor:
    if fn == "lorentzian":
        return 1.0 / (1.0 + 0.5 * z * z)
    if fn == "halfsine":
        return torch.where(z.abs() <= math.pi / 2, torch.cos(z), torch.zeros_like(z))
    if fn == "fullsine":
        return torch.where(z.abs() <= math.pi, 0.5 + torch.cos(z) / 2.0, torch.zeros_like(z))
    if fn == "bisquare":
        return torch.where(z.abs() <= 1.0, (1.0 - z * z) * (1.0 + z * z), torch.zeros_like(z))
    return torch.exp(-0.5 * z * z)


def weights(images: torch.Tensor, theta: torch.Tensor, fn: str = "gaussian", cwin: int = 5,
            range_: float = 1.0) -> torch.Tensor:
    """(K, H, W) weights of (K, H, W, 3) images; theta = (opt, width, W_exp, W_sat, W_con)."""
    opt, width, w_exp, w_sat, w_con = theta
    r, g, b = images[..., 0], images[..., 1], images[..., 2]
    gray = (r + g + b) / 3.0
    z = (gray / range_ - opt) / (width * (FWHM["gaussian"] / FWHM[fn]))
    e = exposure_f(z, fn)
    mx = images.max(dim=-1).values
    mn = images.min(dim=-1).values
    ssum = mx + mn
    den = torch.where(ssum <= 1.0, ssum, 2.0 - ssum)
    sat = torch.where(mx != mn, (mx - mn) / torch.where(mx != mn, den, torch.ones_like(den)), torch.zeros_like(mx))
    K, H, W = gray.shape
    hb = cwin // 2
    win = torch.nn.functional.unfold(gray[:, None], cwin)  # (K, cwin^2, (H-2hb)(W-2hb))
    sd_in = win.std(dim=1, unbiased=True).reshape(K, H - 2 * hb, W - 2 * hb)
    sd = torch.zeros_like(gray)
    sd = sd.clone()
    sd[:, hb:H - hb, hb:W - hb] = sd_in
    return w_exp * e + w_con * sd + w_sat * sat


def to_pyramid(v: torch.Tensor) -> torch.Tensor:
    return torch.where(v >= 0, 1.0 + torch.log1p(v.clamp(min=0.0)), 1.0 / (1.0 - v.clamp(max=0.0)))


def from_pyramid(v: torch.Tensor) -> torch.Tensor:
    return torch.where(v >= 1.0, torch.expm1(v - 1.0), 1.0 - 1.0 / torch.where(v >= 1.0, torch.ones_like(v), v))


def _operators(H: int, W: int, L: int, dev):
    dims = [(H, W)]
    for _ in range(L - 1):
        dims.append(((dims[-1][0] + 1) >> 1, (dims[-1][1] + 1) >> 1))
    Ah = [reduce_matrix(dims[l][0], dev).to_sparse() for l in range(L - 1)]
    Aw = [reduce_matrix(dims[l][1], dev).to_sparse() for l in range(L - 1)]
    Eh = [expand_matrix(dims[l][0], dims[l + 1][0], dev).to_sparse() for l in range(L - 1)]
    Ew = [expand_matrix(dims[l][1], dims[l + 1][1], dev).to_sparse() for l in range(L - 1)]
    return Ah, Aw, Eh, Ew


def _masks(w: torch.Tensor, logits: torch.Tensor) -> torch.Tensor:
    K = w.shape[0]
    wt = w * torch.exp(logits)
    S = wt.sum(dim=0)
    return torch.where(S > 0, wt / torch.where(S > 0, S, torch.ones_like(S)), torch.full_like(wt, 1.0 / K))


def _forward(images: torch.Tensor, logits: torch.Tensor, theta: torch.Tensor, fn: str = "gaussian", cwin: int = 5,
             range_: float = 1.0, levels: int = 0, keep: bool = False):
    """The collapsed level 0 (3, H, W) and, with keep, the weights, masks,
    Laplacians and operators (for the linearised differences below)."""
    K, H, W, _ = images.shape
    L = levels if levels > 0 else num_levels(W, H)
    w = weights(images, theta, fn, cwin, range_)
    m = _masks(w, logits)
    Ah, Aw, Eh, Ew = _operators(H, W, L, images.device)
    G = [to_pyramid(images).permute(0, 3, 1, 2)]  # (K, 3, H, W)
    M = [m[:, None]]
    for l in range(L - 1):
        G.append(separable(Ah[l], G[-1], Aw[l]))
        M.append(separable(Ah[l], M[-1], Aw[l]))
    R, LPs = [], []
    for l in range(L):
        lp = G[l] - separable(Eh[l], G[l + 1], Ew[l]) if l + 1 < L else G[l]
        R.append((lp * M[l]).sum(dim=0))
        if keep:
            LPs.append(lp)
    C = R[L - 1]
    for l in range(L - 2, -1, -1):
        C = R[l] + separable(Eh[l], C, Ew[l])
    parts = dict(w=w, m=m, LP=LPs, ops=(Ah, Aw, Eh, Ew), L=L) if keep else None
    return C, parts


def fuse(images: torch.Tensor, logits: torch.Tensor, theta: torch.Tensor, fn: str = "gaussian", cwin: int = 5,
         range_: float = 1.0, levels: int = 0) -> torch.Tensor:
    """(H, W, 3) fused image of (K, H, W, 3) float64 images."""
    C, _ = _forward(images, logits, theta, fn, cwin, range_, levels)
    return from_pyramid(C).permute(1, 2, 0)


def loss(images, logits, theta, target, **kw) -> torch.Tensor:
    out = fuse(images, logits, theta, **kw)
    return ((out - target) ** 2).mean()


def _phi_difference(p: torch.Tensor, q: torch.Tensor, d: torch.Tensor) -> torch.Tensor:
    """from_pyramid(p) - from_pyramid(q) with d = p - q given exactly:
    e^(q-1) expm1(d) above 1, d / (p q) below, the plain difference where the
    two straddle 1."""
    hi = (p >= 1.0) & (q >= 1.0)
    lo = (p < 1.0) & (q < 1.0)
    one = torch.ones_like(p)
    return torch.where(hi, torch.exp(q - 1.0) * torch.expm1(d),
                       torch.where(lo, d / (torch.where(lo, p, one) * torch.where(lo, q, one)),
                                   from_pyramid(p) - from_pyramid(q)))


def _logit_difference(C: torch.Tensor, parts: dict, logits: torch.Tensor, target: torch.Tensor, k: int, y: int,
                      x: int, step: float) -> float:
    """(L(a + h) - L(a - h)) / 2h for the logit a_k(y, x).  Only the masks of
    pixel (y, x) move, and everything between them and the collapsed level 0
    is linear in the masks: the two mask changes are propagated through the
    mask pyramids, the merge and the collapse on their own (so that the far
    field keeps its significant digits instead of vanishing below the ulp of
    the collapsed values), and the two fused images and the loss difference
    are formed from them without cancellation."""
    Ah, Aw, Eh, Ew = parts["ops"]
    L, LPs = parts["L"], parts["LP"]
    w = parts["w"][:, y, x]
    a = logits[:, y, x].clone()
    m0 = parts["m"][:, y, x]
    dC = []
    for sgn in (1.0, -1.0):
        ak = a.clone()
        ak[k] = a[k] + sgn * step
        dm = _masks(w[:, None, None], ak[:, None, None])[:, 0, 0] - m0
        dM = torch.zeros_like(parts["m"])[:, None]
        dM[:, 0, y, x] = dm
        dR = []
        for l in range(L):
            dR.append((LPs[l] * dM).sum(dim=0))
            if l + 1 < L:
                dM = separable(Ah[l], dM, Aw[l])
        c = dR[L - 1]
        for l in range(L - 2, -1, -1):
            c = dR[l] + separable(Eh[l], c, Ew[l])
        dC.append(c)
    p, q = C + dC[0], C + dC[1]
    dout = _phi_difference(p, q, dC[0] - dC[1])
    t = target.permute(2, 0, 1)
    return float((dout * (from_pyramid(p) + from_pyramid(q) - 2.0 * t)).mean() / (2 * step))


def central_differences(images, logits, theta, target, coords: Sequence, step: float = 1e-6, **kw):
    """FP64 central differences (L(p + h) - L(p - h)) / 2h of the loss at the
    given coordinates: ("theta", i) or ("logit", k, y, x).  The difference of
    the two means of squares is formed per pixel as (a - b)(a + b - 2t) with
    a, b the two fused images; for a logit coordinate the change of a - b is
    propagated on its own (_logit_difference), because one pixel's logit
    moves most pixels of a large image by less than their ulp."""
    out = []
    with torch.no_grad():
        C = parts = None
        for c in coords:
            if c[0] == "logit":
                if parts is None:
                    C, parts = _forward(images, logits, theta, keep=True, **kw)
                out.append(_logit_difference(C, parts, logits, target, c[1], c[2], c[3], step))
                continue
            tp, tm = theta.clone(), theta.clone()
            tp[c[1]] += step
            tm[c[1]] -= step
            a = fuse(images, logits, tp, **kw)
            b = fuse(images, logits, tm, **kw)
            out.append(float(((a - b) * (a + b - 2.0 * target)).mean() / (2 * step)))
    return np.array(out)
