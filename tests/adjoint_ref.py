"""Oracle-side discrete adjoint (FP64, direct solves) used to check the GPU adjoint."""
import ctypes as C

import numpy as np
import scipy.sparse.linalg as spla

from oracle import oracle as O


def oracle_param_derivs(prob, x):
    L = O.lib()
    nc = prob.cell_X.shape[0]
    xc = np.ascontiguousarray(prob.cell_values(x))
    dg = np.zeros((nc, 129)); dc = np.zeros((nc, 129)); fz = np.zeros((nc, 27))
    sf, k1 = O._c_fluid(prob.fluid)
    sc, k2 = O._c_facets(prob.facets)
    L.orc_param_derivs(C.c_int64(nc), O._dp(prob.cell_X), O._dp(xc), C.byref(sf), C.byref(sc), O._dp(dg),
                       O._dp(dc), O._dp(fz))
    g = prob.gdofs
    m = g >= 0
    dR_dgamma = np.bincount(g[m], weights=dg[m], minlength=prob.ndofs)
    dR_dcw = np.bincount(g[m], weights=dc[m], minlength=prob.ndofs)
    return dR_dgamma, dR_dcw, fz


def oracle_param_derivs_ab(prob, x):
    """∂R/∂α and ∂R/∂β (global vectors) at x."""
    L = O.lib()
    nc = prob.cell_X.shape[0]
    xc = np.ascontiguousarray(prob.cell_values(x))
    da = np.zeros((nc, 129)); db = np.zeros((nc, 129))
    sf, k1 = O._c_fluid(prob.fluid)
    L.orc_param_derivs_ab(C.c_int64(nc), O._dp(prob.cell_X), O._dp(xc), C.byref(sf), O._dp(da), O._dp(db))
    g = prob.gdofs
    m = g >= 0
    return (np.bincount(g[m], weights=da[m], minlength=prob.ndofs),
            np.bincount(g[m], weights=db[m], minlength=prob.ndofs))


def oracle_adjoint_ab(prob, lam, x):
    """dJ/dα and dJ/dβ from the adjoint vector λ at x."""
    dRa, dRb = oracle_param_derivs_ab(prob, x)
    return -lam @ dRa, -lam @ dRb


def oracle_adjoint(prob, dm, x, dJdx, gauge):
    """dJ/dγ, dJ/dcw, dJ/df_z(cell) at the solution x."""
    _, A = prob.residual_jacobian(x)
    keep = np.ones(prob.ndofs, bool)
    keep[list(gauge)] = False
    idx = np.nonzero(keep)[0]
    lam = np.zeros(prob.ndofs)
    lam[idx] = spla.spsolve(A[idx][:, idx].T.tocsc(), dJdx[idx])
    dRg, dRc, fz = oracle_param_derivs(prob, x)
    gd = dm.global_cell_dofs()[:, 54:81]
    lz = np.where(gd >= 0, lam[np.maximum(gd, 0)], 0.0)
    return -lam @ dRg, -lam @ dRc, np.sum(lz * fz, 1), lam
