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
(flag 0).  A wall cell holds the rest state w_i * rho_w, rho_w the mean
predicted density of its fluid neighbours (1 when it has none).
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
    f = np.zeros((ny, nx, 9))
    for y in range(ny):
        for x in range(nx):
            if not fluid[y, x]:
                acc, cnt = 0.0, 0
                for i in range(1, 9):
                    xx, yy = x + CX[i], y + CY[i]
                    if 0 <= xx < nx and 0 <= yy < ny and fluid[yy, xx]:
                        acc += rho[yy, xx]
                        cnt += 1
                f[y, x] = W * (acc / cnt if cnt else 1.0)
                continue
            u = np.array([ux[y, x], uy[y, x]])
            r = rho[y, x]
            cu = CX * u[0] + CY * u[1]
            f[y, x] = W * r * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * (u @ u))
            if with_neq:
                xm, xp = max(x - 1, 0), min(x + 1, nx - 1)
                ym, yp = max(y - 1, 0), min(y + 1, ny - 1)
                dxu = (ux[y, xp] - ux[y, xm]) / (xp - xm)
                dxv = (uy[y, xp] - uy[y, xm]) / (xp - xm)
                dyu = (ux[yp, x] - ux[ym, x]) / (yp - ym)
                dyv = (uy[yp, x] - uy[ym, x]) / (yp - ym)
                sxy = 0.5 * (dxv + dyu)
                qs = (CX * CX - 1 / 3) * dxu + (CY * CY - 1 / 3) * dyv + 2.0 * CX * CY * sxy
                f[y, x] -= tau * W * r * 3.0 * qs
    return f.reshape(ny * nx, 9)
