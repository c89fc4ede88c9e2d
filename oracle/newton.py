"""FP64 restatement of the reference's Newton driver and line search.

TEST INFRASTRUCTURE ONLY (the checker for the GPU solver; see oracle.py).

* newtons_method_bisection: include/optimization_gradient_based.h:43-110
* linesearch_backtracking_bisection: src/linesearch_backtracking_bisection.cpp:5-31
* search_direction_newton_sparse: src/search_direction_newton_sparse.cpp:5-26, with
  scipy's SuperLU in place of Eigen::SparseLU (both direct LU solves).
* implicit-Euler objective in velocity form: matlab/examples/implicit_integration.m:69-83.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import oracle as o

CONVERGED, MAX_ITERATIONS_REACHED = 0, 1


def linesearch_backtracking_bisection(x, d, f, g, max_iterations, alpha, c, p):
    it = 0
    fx = f(x)
    while f(x + alpha * d) > fx + c * (g @ d) and it < max_iterations:
        alpha *= p
        it += 1
    x += alpha * d
    return MAX_ITERATIONS_REACHED if it == max_iterations else CONVERGED


def search_direction_newton_sparse(g, H):
    try:
        d = -spla.spsolve(sp.csc_matrix(H), g)
    except Exception:
        return None
    return d if np.all(np.isfinite(d)) else None


def newtons_method_bisection(x, f, grad, hess, gradient_tol=1e-3, max_iterations=100, max_iterations_ls=100,
                             alpha=1.0, c=1e-8, p=0.5, relative=False):
    """Returns (status, iterations). relative=True stops on ||g|| <= tol ||g_0||
    (the configs' criterion) instead of the reference's absolute g.g < tol^2."""
    count = 0
    g0 = None
    while True:
        g = grad(x)
        gg = g @ g
        if g0 is None:
            g0 = np.sqrt(gg)
        if (np.sqrt(gg) <= gradient_tol * g0) if relative else (gg < gradient_tol * gradient_tol):
            return CONVERGED, count
        d = search_direction_newton_sparse(g, hess(x))
        if d is None:
            raise RuntimeError("Computing search direction failed in newtons method")
        linesearch_backtracking_bisection(x, d, f, g, max_iterations_ls, alpha, c, p)
        count += 1
        if count > max_iterations:
            return MAX_ITERATIONS_REACHED, count


class Objective:
    """f(x) = mass_coeff (x^T M x / 2 - x^T M x_hat) + Psi(q_base + scale x) - force_scale x^T f_ext,
    restricted to the free vertices through P (fixed_point_constraint_matrix)."""

    def __init__(self, model, V, E, params, density, q_base, x_hat, f_ext, pinned, mass_coeff, scale, force_scale,
                 psd_tol=None):
        self.model, self.V, self.E = model, V, E
        self.nV = len(V)
        self.dphi = o.dphi_dX(V, E)
        self.vol = o.volume(V, E)
        self.params = params
        self.M = o.mass_matrix(self.nV, E, density, self.vol)
        fixed = np.nonzero(pinned)[0].astype(np.int32)
        self.P = o.fixed_point_constraint_matrix(self.nV, fixed)
        self.q_base = np.zeros(3 * self.nV) if q_base is None else q_base
        self.x_hat = np.zeros(3 * self.nV) if x_hat is None else x_hat
        self.f_ext = np.zeros(3 * self.nV) if f_ext is None else f_ext
        self.mc, self.s, self.fs = mass_coeff, scale, force_scale
        self.psd_tol = psd_tol

    def full(self, xr):
        return self.P.T @ xr

    def f(self, xr):
        x = self.full(xr)
        q = self.q_base + self.s * x
        e = o.tetmesh_q(self.model, self.E, q, self.dphi, self.vol, self.params)
        e += self.mc * (0.5 * x @ (self.M @ x) - x @ (self.M @ self.x_hat))
        return e - self.fs * (x @ self.f_ext)

    def grad(self, xr):
        x = self.full(xr)
        q = self.q_base + self.s * x
        g = self.s * o.tetmesh_dq(self.model, self.nV, self.E, q, self.dphi, self.vol, self.params)
        g += self.mc * (self.M @ (x - self.x_hat)) - self.fs * self.f_ext
        return self.P @ g

    def hess(self, xr):
        x = self.full(xr)
        q = self.q_base + self.s * x
        K = o.tetmesh_dq2(self.model, self.nV, self.E, q, self.dphi, self.vol, self.params, psd_tol=self.psd_tol)
        return (self.P @ (self.mc * self.M + self.s * self.s * K) @ self.P.T).tocsr()
