"""FP64 references for the adjoint tests (test code only).

L(rho) = g2 |eps_2| + g3 |eps_3| + <g_rho, rho>, eps_n = |Z_n| / D_n with
Z_n = sum_M z^n rho, D_n = sum_M |z|^n rho over the hot-spot region M and z
about the density's centre of mass (over all cells): the r^n-weighted
eccentricities of MakeDensity::dumpEccentricities
(src/MakeDensity.cpp:2244-2511).  ``objective`` evaluates L; ``adjoint_grid``
is the closed-form dL/d rho the adjoint kernel forms on the GPU;
``fd_gradient`` differentiates L(rho(w, alpha)) by central differences with
the oracle's frozen-structure density (smco_event_density_frozen).
"""
import numpy as np


def _coords(nx, ny, xmin, ymin, dx, dy):
    x = xmin + np.arange(nx) * dx
    y = ymin + np.arange(ny) * dy
    return np.meshgrid(x, y, indexing="ij")


def eps_n(rho, mask, X, Y):
    tot = rho.sum()
    xc, yc = (X * rho).sum() / tot, (Y * rho).sum() / tot
    z = (X - xc) + 1j * (Y - yc)
    out = []
    for n in (2, 3):
        zm, rm = z[mask], rho[mask]
        out.append(abs((zm ** n * rm).sum()) / ((np.abs(zm) ** n * rm).sum() + 1e-15))
    return np.array(out)


def objective(rho, mask, X, Y, g_eps, g_rho):
    L = 0.0
    if g_eps is not None:
        L += float(np.dot(g_eps, eps_n(rho, mask, X, Y)))
    if g_rho is not None:
        L += float((g_rho.astype(np.float64) * rho).sum())
    return L


def adjoint_grid(rho, mask, X, Y, g_eps, g_rho):
    """dL/d rho(c) including the centre of mass's dependence on rho."""
    tot = rho.sum()
    xc, yc = (X * rho).sum() / tot, (Y * rho).sum() / tot
    z = (X - xc) + 1j * (Y - yc)
    r = np.abs(z)
    lam = np.zeros_like(rho) if g_rho is None else g_rho.astype(np.float64).copy()
    if g_eps is None:
        return lam
    cx = cy = 0.0
    for q, n in enumerate((2, 3)):
        m = mask
        Z = (z[m] ** n * rho[m]).sum()
        D = (r[m] ** n * rho[m]).sum() + 1e-15
        U = (n * z[m] ** (n - 1) * rho[m]).sum()
        V = (n * r[m] ** (n - 2) * z[m] * rho[m]).sum()
        A = g_eps[q] / (abs(Z) * D)
        B = -g_eps[q] * abs(Z) / D ** 2
        lam[m] += A * (np.conj(Z) * z[m] ** n).real + B * r[m] ** n
        cx += A * (np.conj(Z) * -U).real + B * -V.real
        cy += A * (np.conj(Z) * (-1j * U)).real + B * -V.imag
    lam += (cx * (X - xc) + cy * (Y - yc)) / tot
    return lam


def fd_gradient(ev, mask, X, Y, w, alpha, g_eps, g_rho, h=1e-4):
    """Central differences (step h) of L in w and alpha, FP64."""
    def L(ww, aa):
        return objective(ev.density_frozen(ww, aa), mask, X, Y, g_eps, g_rho)
    dw = (L(w + h, alpha) - L(w - h, alpha)) / (2 * h)
    da = (L(w, alpha + h) - L(w, alpha - h)) / (2 * h)
    return np.array([dw, da])


def grid_coords(vals, nx, ny):
    return _coords(nx, ny, -vals["maxx"], -vals["maxy"], vals["dx"], vals["dy"])
