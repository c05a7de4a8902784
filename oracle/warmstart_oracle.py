"""FP64 numpy restatement of the warm-start population reconstruction
(kel_batch_warm_start).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the product package.

The reference has no warm start (its drivers start from rest equilibrium,
examples/stdkr_2d_bgk/init.hpp:16-54); the equilibrium restated here is the
reference's second-order BGK equilibrium (modules/core/c++/equilibrium.hpp:27-45)
in exact arithmetic, and the non-equilibrium part is the first-order
Chapman-Enskog population
    f_neq_i = -(tau w_i rho / cs^2) Q_i : grad u,   Q_i = c_i c_i - cs^2 I,
with grad u from central differences (one-sided at the channel ends) of the
predicted velocity, taken as zero in wall cells (flag 1) and outside cells
(flag 0).  A wall cell holds, in each slot i whose source x - c_i is fluid,
that cell's post-collision population f_eq + (1 - 1/tau) f_neq, and in the
other slots the rest state w_i * rho_w, rho_w the mean predicted density of
its fluid neighbours (1 when it has none).
"""
from __future__ import annotations

import numpy as np

# D2Q9 in the library's (and the reference's) direction order
CX = np.array([0, -1, 1, 0, 0, -1, 1, -1, 1])
CY = np.array([0, 0, 0, -1, 1, -1, 1, 1, -1])
W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36])


def warm_start_populations(flags, pred, scale, offset, tau, with_neq=True):
    """flags (ny, nx) uint8, pred (ny, nx, 3) -> populations (ny*nx, 9) AoS,
    x fastest, float64."""
    flags = np.asarray(flags).reshape(pred.shape[:2])
    ny, nx = flags.shape
    fluid = (flags != 1) & (flags != 0)
    phys = pred.astype(np.float64) * np.asarray(scale, np.float64) + np.asarray(offset, np.float64)
    ux = np.where(fluid, phys[..., 0], 0.0)
    uy = np.where(fluid, phys[..., 1], 0.0)
    rho = phys[..., 2]

    def pops(x, y, fac):
        u = np.array([ux[y, x], uy[y, x]])
        r = rho[y, x]
        cu = CX * u[0] + CY * u[1]
        f = W * r * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * (u @ u))
        if with_neq:
            xm, xp = max(x - 1, 0), min(x + 1, nx - 1)
            ym, yp = max(y - 1, 0), min(y + 1, ny - 1)
            dxu = (ux[y, xp] - ux[y, xm]) / (xp - xm)
            dxv = (uy[y, xp] - uy[y, xm]) / (xp - xm)
            dyu = (ux[yp, x] - ux[ym, x]) / (yp - ym)
            dyv = (uy[yp, x] - uy[ym, x]) / (yp - ym)
            qs = (CX * CX - 1 / 3) * dxu + (CY * CY - 1 / 3) * dyv + CX * CY * (dxv + dyu)
            f = f - fac * tau * W * r * 3.0 * qs
        return f

    post = 1.0 - 1.0 / tau
    f = np.zeros((ny, nx, 9))
    for y in range(ny):
        for x in range(nx):
            if fluid[y, x]:
                f[y, x] = pops(x, y, 1.0)
                continue
            acc, cnt = 0.0, 0
            for i in range(1, 9):
                xx, yy = x + CX[i], y + CY[i]
                if 0 <= xx < nx and 0 <= yy < ny and fluid[yy, xx]:
                    acc += rho[yy, xx]
                    cnt += 1
            f[y, x] = W * (acc / cnt if cnt else 1.0)
            for i in range(1, 9):
                xs, ys = x - CX[i], y - CY[i]
                if 0 <= xs < nx and 0 <= ys < ny and fluid[ys, xs]:
                    f[y, x, i] = pops(xs, ys, post)[i]
    return f.reshape(ny * nx, 9)


def unet_input(mask, u_max, tau):
    """FP64 restatement of the network input planes (kel_unet_make_input):
    mask (n, H, W) uint8 (1 = solid), u_max / tau (n,) -> (n, H, W, 16)."""
    mask = np.asarray(mask)
    n, H, W = mask.shape
    hin = float(H - 2 if H > 2 else H)
    out = np.zeros((n, H, W, 16))
    for b in range(n):
        m = mask[b]
        openf = np.minimum((m == 0).sum(axis=0) / hin, 1.0)
        h3 = np.zeros(W)
        for x in range(W):
            run = 0
            for y in range(H):
                if m[y, x] == 0:
                    run += 1
                else:
                    h3[x] += run ** 3
                    run = 0
            h3[x] += run ** 3
        R = np.cumsum((1.0 / np.maximum(openf, 0.125) ** 3)[::-1])[::-1] / W
        S = np.cumsum((1.0 / np.maximum(h3, 1.0))[::-1])[::-1]  # lubrication pressure, suffix sums
        PL = S / S[0]
        out[b, :, :, 0] = m
        out[b, :, :, 1] = u_max[b] / 0.08
        out[b, :, :, 2] = (tau[b] - 0.55) / 0.45
        out[b, :, :, 3] = np.arange(H)[:, None] / (H - 1)
        out[b, :, :, 4] = np.arange(W)[None, :] / (W - 1)
        for x in range(W):
            y = 0
            while y < H:
                if m[y, x]:
                    y += 1
                    continue
                lo = y
                while y + 1 < H and m[y + 1, x] == 0:
                    y += 1
                hi = y
                h = hi - lo + 1
                for yy in range(lo, hi + 1):
                    sp = (yy - lo + 0.5) / h
                    shape = 4 * sp * (1 - sp)
                    out[b, yy, x, 5] = openf[x]
                    out[b, yy, x, 6] = R[x]
                    out[b, yy, x, 7] = h / hin
                    out[b, yy, x, 8] = shape
                    out[b, yy, x, 9] = 0.5 * min(hin * h * h / max(h3[x], 1.0) * shape, 8.0)
                    out[b, yy, x, 10] = PL[x]
                y += 1
    return out
