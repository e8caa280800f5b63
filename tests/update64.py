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
