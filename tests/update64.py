"""FP64 PyTorch re-expression of one image update with the NNF held fixed,
for checking the adjoint kernels: out = U(u; lambda, sigma) with orig = u.

NL-means follows patch_non_local_means.cpp:23-100 (weights indexed from the
clipped window corner, confidence inside the domain only).  NL-Poisson
follows patch_non_local_poisson.cpp:36-232 with the coefficient gather of
the CUDA kernels (every pixel collects from the centres whose window holds
it), the system (lambda S - (1 - lambda) div S grad) delta = b on the hole
and out = u + delta.  Gaussian patch weights as gaussian_weights.cpp:19-79:
exp(-r^2 / (2 sigma^2)) normalised by their sum, here in double.

Differentiable in u, lambda and sigma with a dense solve (small sizes);
`solver="sparse"` solves with scipy in FP64 instead (no autograd) for
finite differences at full size.  Test infrastructure only.
"""
from __future__ import annotations

import numpy as np
import torch


def patch_weights(sigma, px, py):
    hx, hy = px // 2, py // 2
    ky, kx = torch.meshgrid(torch.arange(py, dtype=torch.float64) - hy, torch.arange(px, dtype=torch.float64) - hx,
                            indexing="ij")
    e = torch.exp(-(kx * kx + ky * ky) / (2.0 * sigma * sigma))
    return (e / e.sum()).reshape(-1)


def _forward_diff(u):
    gx = torch.zeros_like(u)
    gy = torch.zeros_like(u)
    gx[:, :-1] = u[:, 1:] - u[:, :-1]
    gy[:-1, :] = u[1:, :] - u[:-1, :]
    return gx, gy


def means(u, sigma, nnf, dom, conf, px=9, py=9):
    """u: (H, W, C) float64 tensor; nnf: (H, W, 2) int array; dom: (H, W)
    bool array; conf: (H, W) array or None."""
    H, W, C = u.shape
    hx, hy = px // 2, py // 2
    g = patch_weights(sigma, px, py)
    ys, xs = np.nonzero(dom)
    num = torch.zeros((len(ys), C), dtype=torch.float64)
    den = torch.zeros(len(ys), dtype=torch.float64)
    xa, ya = np.maximum(xs - hx, 0), np.maximum(ys - hy, 0)
    xb, yb = np.minimum(xs + hx, W - 1), np.minimum(ys + hy, H - 1)
    for dy in range(-hy, hy + 1):
        for dx in range(-hx, hx + 1):
            ii, jj = xs + dx, ys + dy
            inside = (ii >= xa) & (ii <= xb) & (jj >= ya) & (jj <= yb)
            iic, jjc = np.clip(ii, 0, W - 1), np.clip(jj, 0, H - 1)
            q = nnf[jjc, iic]
            qx, qy = q[:, 0] + xs - iic, q[:, 1] + ys - jjc
            ok = inside & (q[:, 0] != -1) & (qx >= 0) & (qy >= 0) & (qx < W) & (qy < H)
            if not ok.any():
                continue
            k = torch.from_numpy(((jjc - ya) * px + (iic - xa))[ok])
            w = g[k]
            if conf is not None:
                cf = np.where(dom[jjc, iic], conf[jjc, iic], 1.0)[ok]
                w = w * torch.from_numpy(cf.astype(np.float64))
            idx = torch.from_numpy(np.nonzero(ok)[0])
            den = den.index_add(0, idx, w)
            num = num.index_add(0, idx, w[:, None] * u[qy[ok], qx[ok]])
    out = u.clone()
    has = den > 0
    sel = torch.from_numpy(np.nonzero(has.numpy())[0])
    out[ys[has.numpy()], xs[has.numpy()]] = num[sel] / den[sel][:, None]
    return out


def poisson_coefficients(u, sigma, nnf, ext, conf, px=9, py=9):
    """S (H, W), U, GX, GY (H, W, C): every pixel q collects
    w = conf(c) g(q - c) and u, gx, gy at n = nnf(c) + q - c from each
    extended-domain centre c of its window with n in the image."""
    H, W, C = u.shape
    hx, hy = px // 2, py // 2
    g = patch_weights(sigma, px, py)
    gx, gy = _forward_diff(u)
    S = torch.zeros((H, W), dtype=torch.float64)
    U = torch.zeros((H, W, C), dtype=torch.float64)
    GX = torch.zeros_like(U)
    GY = torch.zeros_like(U)
    qy, qx = np.mgrid[0:H, 0:W]
    for dy in range(-hy, hy + 1):
        for dx in range(-hx, hx + 1):
            cx, cy = qx - dx, qy - dy
            ok = (cx >= 0) & (cy >= 0) & (cx < W) & (cy < H)
            cxc, cyc = np.clip(cx, 0, W - 1), np.clip(cy, 0, H - 1)
            ok &= ext[cyc, cxc] != 0
            nb = nnf[cyc, cxc]
            nx, ny = nb[..., 0] + dx, nb[..., 1] + dy
            ok &= (nx >= 0) & (ny >= 0) & (nx < W) & (ny < H)
            if not ok.any():
                continue
            k = (dy + hy) * px + (dx + hx)
            wv = torch.zeros((H, W), dtype=torch.float64)
            cfv = np.ones((H, W)) if conf is None else conf[cyc, cxc]
            wv[ok] = g[k] * torch.from_numpy(cfv[ok].astype(np.float64))
            nxc, nyc = np.clip(nx, 0, W - 1), np.clip(ny, 0, H - 1)
            S = S + wv
            U = U + wv[..., None] * u[nyc, nxc]
            GX = GX + wv[..., None] * gx[nyc, nxc]
            GY = GY + wv[..., None] * gy[nyc, nxc]
    return S, U, GX, GY


def poisson(u, lam, sigma, nnf, dom, ext, conf, px=9, py=9, lam_channels=None, solver="dense"):
    """NL-Poisson step (NL-depth when lam_channels gives a per-channel
    lambda tensor).  Returns the updated image."""
    H, W, C = u.shape
    S, U, GX, GY = poisson_coefficients(u, sigma, nnf, ext, conf, px, py)
    ys, xs = np.nonzero(dom)
    nh = len(ys)
    index = -np.ones((H, W), dtype=np.int64)
    index[ys, xs] = np.arange(nh)
    out = u.clone()
    for c in range(C):
        lc = lam if lam_channels is None else lam_channels[c]
        oml = 1.0 - lc
        o = u[..., c]
        Sk = S[ys, xs]
        D = torch.zeros(nh, dtype=torch.float64)
        D = D + torch.where(torch.from_numpy(xs != W - 1), GX[ys, xs, c], torch.zeros(nh, dtype=torch.float64))
        D = D - torch.where(torch.from_numpy(xs != 0), GX[ys, np.maximum(xs - 1, 0), c],
                            torch.zeros(nh, dtype=torch.float64))
        D = D + torch.where(torch.from_numpy(ys != H - 1), GY[ys, xs, c], torch.zeros(nh, dtype=torch.float64))
        D = D - torch.where(torch.from_numpy(ys != 0), GY[np.maximum(ys - 1, 0), xs, c],
                            torch.zeros(nh, dtype=torch.float64))
        b = lc * U[ys, xs, c] - oml * D - lc * Sk * o[ys, xs]
        rows, cols, vals = [np.arange(nh)], [np.arange(nh)], [lc * Sk]
        diag_extra = torch.zeros(nh, dtype=torch.float64)
        for (ddx, ddy, s_of) in ((0, -1, "up"), (-1, 0, "left"), (0, 1, "down"), (1, 0, "right")):
            nx, ny = xs + ddx, ys + ddy
            inside = (nx >= 0) & (ny >= 0) & (nx < W) & (ny < H)
            if s_of == "up":
                s = torch.where(torch.from_numpy(inside), S[np.maximum(ny, 0), xs], torch.zeros(nh, dtype=torch.float64))
            elif s_of == "left":
                s = torch.where(torch.from_numpy(inside), S[ys, np.maximum(nx, 0)], torch.zeros(nh, dtype=torch.float64))
            else:
                s = torch.where(torch.from_numpy(inside), Sk, torch.zeros(nh, dtype=torch.float64))
            nxc, nyc = np.clip(nx, 0, W - 1), np.clip(ny, 0, H - 1)
            b = b + oml * s * (o[nyc, nxc] - o[ys, xs])
            diag_extra = diag_extra + oml * s
            nbk = np.where(inside, index[nyc, nxc], -1)
            m = nbk >= 0
            rows.append(np.nonzero(m)[0])
            cols.append(nbk[m])
            vals.append(-oml * s[torch.from_numpy(np.nonzero(m)[0])])
        vals[0] = vals[0] + diag_extra
        r = torch.from_numpy(np.concatenate(rows))
        cc = torch.from_numpy(np.concatenate(cols))
        v = torch.cat(vals)
        if solver == "dense":
            A = torch.zeros((nh, nh), dtype=torch.float64).index_put((r, cc), v, accumulate=True)
            delta = torch.linalg.solve(A, b)
        else:
            import scipy.sparse as sp
            import scipy.sparse.linalg as spl
            A = sp.csr_matrix((v.detach().numpy(), (r.numpy(), cc.numpy())), shape=(nh, nh))
            delta = torch.from_numpy(spl.spsolve(A.tocsc(), b.detach().numpy()))
        out[ys, xs, c] = o[ys, xs] + delta
    return out


# --------------------------------------------------------------- fast path
# The same FP64 expressions, vectorised for full-size finite differences
# (no autograd): the gather structure of a case -- which centre and which
# source pixel every (pixel, tap) pair reads -- is built once, and each
# evaluation is a few weighted bincounts and one sparse factorisation.
class Plan:
    """Gather structure of one (nnf, dom, ext, conf) case."""

    def __init__(self, nnf, dom, ext, conf, px=9, py=9):
        H, W = dom.shape
        self.H, self.W, self.px, self.py = H, W, px, py
        hx, hy = px // 2, py // 2
        self.dom = np.asarray(dom, bool)
        conf = np.ones((H, W)) if conf is None else np.asarray(conf, np.float64)
        ys, xs = np.nonzero(self.dom)
        self.ys, self.xs = ys, xs
        nh = len(ys)
        self.index = -np.ones((H, W), np.int64)
        self.index[ys, xs] = np.arange(nh)
        # NL-means: per hole pixel, the window pixels (ii, jj) with a match
        mi, mk, msrc, ms = [], [], [], []
        xa, ya = np.maximum(xs - hx, 0), np.maximum(ys - hy, 0)
        xb, yb = np.minimum(xs + hx, W - 1), np.minimum(ys + hy, H - 1)
        for dy in range(-hy, hy + 1):
            for dx in range(-hx, hx + 1):
                ii, jj = xs + dx, ys + dy
                inside = (ii >= xa) & (ii <= xb) & (jj >= ya) & (jj <= yb)
                iic, jjc = np.clip(ii, 0, W - 1), np.clip(jj, 0, H - 1)
                q = nnf[jjc, iic]
                qx, qy = q[:, 0] + xs - iic, q[:, 1] + ys - jjc
                ok = inside & (q[:, 0] != -1) & (qx >= 0) & (qy >= 0) & (qx < W) & (qy < H)
                k = (jjc - ya) * px + (iic - xa)
                cf = np.where(self.dom[jjc, iic], conf[jjc, iic], 1.0)
                mi.append(np.nonzero(ok)[0])
                mk.append(k[ok])
                msrc.append(qy[ok] * W + qx[ok])
                ms.append(cf[ok])
        self.m_i = np.concatenate(mi)
        self.m_k = np.concatenate(mk)
        self.m_src = np.concatenate(msrc)
        self.m_conf = np.concatenate(ms)
        # NL-Poisson: per pixel q (every pixel), the taps with a valid centre
        qy_, qx_ = np.mgrid[0:H, 0:W]
        pi, pk, psrc, pc = [], [], [], []
        ext = np.asarray(ext) != 0
        for dy in range(-hy, hy + 1):
            for dx in range(-hx, hx + 1):
                cx, cy = qx_ - dx, qy_ - dy
                ok = (cx >= 0) & (cy >= 0) & (cx < W) & (cy < H)
                cxc, cyc = np.clip(cx, 0, W - 1), np.clip(cy, 0, H - 1)
                ok &= ext[cyc, cxc]
                nb = nnf[cyc, cxc]
                nx, ny = nb[..., 0] + dx, nb[..., 1] + dy
                ok &= (nx >= 0) & (ny >= 0) & (nx < W) & (ny < H)
                sel = np.nonzero(ok.reshape(-1))[0]
                pi.append(sel)
                pk.append(np.full(len(sel), (dy + hy) * px + (dx + hx), np.int64))
                psrc.append((ny * W + nx).reshape(-1)[sel])
                pc.append(conf[cyc, cxc].reshape(-1)[sel])
        self.p_i = np.concatenate(pi)
        self.p_k = np.concatenate(pk)
        self.p_src = np.concatenate(psrc)
        self.p_conf = np.concatenate(pc)

    def weights(self, sigma):
        return patch_weights(float(sigma), self.px, self.py).numpy()


def means_fast(u, sigma, plan):
    """NL-means of `means` on the plan's case; u: (H, W, C) float64 array."""
    H, W, C = u.shape
    g = plan.weights(sigma)
    w = g[plan.m_k] * plan.m_conf
    nh = len(plan.ys)
    den = np.bincount(plan.m_i, weights=w, minlength=nh)
    flat = u.reshape(-1, C)
    out = u.copy()
    has = den > 0
    for c in range(C):
        num = np.bincount(plan.m_i, weights=w * flat[plan.m_src, c], minlength=nh)
        vals = out[plan.ys, plan.xs, c]
        vals[has] = num[has] / den[has]
        out[plan.ys, plan.xs, c] = vals
    return out


def poisson_fast(u, lam, sigma, plan, lam_channels=None):
    """NL-Poisson / NL-depth of `poisson` on the plan's case (direct sparse
    solve, one factorisation per distinct lambda)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    H, W, C = u.shape
    n = H * W
    g = plan.weights(sigma)
    w = g[plan.p_k] * plan.p_conf
    flat = u.reshape(-1, C)
    gx = np.zeros_like(u)
    gy = np.zeros_like(u)
    gx[:, :-1] = u[:, 1:] - u[:, :-1]
    gy[:-1, :] = u[1:, :] - u[:-1, :]
    gxf, gyf = gx.reshape(-1, C), gy.reshape(-1, C)
    S = np.bincount(plan.p_i, weights=w, minlength=n).reshape(H, W)
    ys, xs = plan.ys, plan.xs
    nh = len(ys)
    Sk = S[ys, xs]
    links = []
    for (ddx, ddy, kind) in ((0, -1, "up"), (-1, 0, "left"), (0, 1, "down"), (1, 0, "right")):
        nx, ny = xs + ddx, ys + ddy
        inside = (nx >= 0) & (ny >= 0) & (nx < W) & (ny < H)
        if kind == "up":
            s = np.where(inside, S[np.maximum(ny, 0), xs], 0.0)
        elif kind == "left":
            s = np.where(inside, S[ys, np.maximum(nx, 0)], 0.0)
        else:
            s = np.where(inside, Sk, 0.0)
        nxc, nyc = np.clip(nx, 0, W - 1), np.clip(ny, 0, H - 1)
        links.append((s, nxc, nyc, np.where(inside, plan.index[nyc, nxc], -1)))
    out = u.copy()
    factors = {}
    for c in range(C):
        lc = float(lam if lam_channels is None else lam_channels[c])
        oml = 1.0 - lc
        U = np.bincount(plan.p_i, weights=w * flat[plan.p_src, c], minlength=n).reshape(H, W)
        GX = np.bincount(plan.p_i, weights=w * gxf[plan.p_src, c], minlength=n).reshape(H, W)
        GY = np.bincount(plan.p_i, weights=w * gyf[plan.p_src, c], minlength=n).reshape(H, W)
        o = u[..., c]
        D = np.where(xs != W - 1, GX[ys, xs], 0.0) - np.where(xs != 0, GX[ys, np.maximum(xs - 1, 0)], 0.0)
        D += np.where(ys != H - 1, GY[ys, xs], 0.0) - np.where(ys != 0, GY[np.maximum(ys - 1, 0), xs], 0.0)
        b = lc * U[ys, xs] - oml * D - lc * Sk * o[ys, xs]
        for s, nxc, nyc, _ in links:
            b = b + oml * s * (o[nyc, nxc] - o[ys, xs])
        if lc not in factors:
            rows, cols, vals = [np.arange(nh)], [np.arange(nh)], [lc * Sk + oml * sum(l[0] for l in links)]
            for s, _, _, nbk in links:
                m = nbk >= 0
                rows.append(np.nonzero(m)[0])
                cols.append(nbk[m])
                vals.append(-oml * s[m])
            A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nh, nh))
            factors[lc] = spl.splu(A)
        out[ys, xs, c] = o[ys, xs] + factors[lc].solve(b)
    return out
