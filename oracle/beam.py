"""CPU oracle of the beam FE model (TEST INFRASTRUCTURE ONLY).

Restates src/fluxvortex/beam_fe.py of the FLUXVortex project in NumPy, FP64:
  * element matrices: Hermite cubic bending stiffness and consistent mass
    (beam_fe.py:87-105), linear torsion stiffness and mass (:107-120), and the
    bending-torsion coupling mass from the CG offset by 3-point Gauss
    quadrature on [0, 1] (:122-172);
  * assembly with per-node DOF [w, dw/dy, theta] (:174-213);
  * cantilever boundary condition: the root node's three DOF removed
    (:215-229);
  * Rayleigh damping C = (2 zeta / omega_1) K with omega_1 from the reduced
    generalised eigenproblem (:64-74);
  * Newmark average acceleration (beta = 1/4, gamma = 1/2) with a dense solve
    of the effective stiffness (:231-277);
  * linear distribution of station forces and moments to the nodes
    (:316-351).
Pinned by tests/golden/beam_goland.npz (generated by importing the
reference's BeamFE).
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import eigh


def element_matrices(EI, GJ, m, Ip, xc, Le):
    L = Le
    Kb = EI / L ** 3 * np.array([[12, 6 * L, -12, 6 * L],
                                 [6 * L, 4 * L ** 2, -6 * L, 2 * L ** 2],
                                 [-12, -6 * L, 12, -6 * L],
                                 [6 * L, 2 * L ** 2, -6 * L, 4 * L ** 2]])
    Mb = m * L / 420 * np.array([[156, 22 * L, 54, -13 * L],
                                 [22 * L, 4 * L ** 2, 13 * L, -3 * L ** 2],
                                 [54, 13 * L, 156, -22 * L],
                                 [-13 * L, -3 * L ** 2, -22 * L, 4 * L ** 2]])
    Kt = GJ / L * np.array([[1, -1], [-1, 1]])
    Mt = Ip * L / 6 * np.array([[2, 1], [1, 2]])
    g = np.array([0.5 - 0.5 * np.sqrt(0.6), 0.5, 0.5 + 0.5 * np.sqrt(0.6)])
    w = np.array([5.0, 8.0, 5.0]) / 18.0
    Nb = np.array([1 - 3 * g ** 2 + 2 * g ** 3, L * (g - 2 * g ** 2 + g ** 3),
                   3 * g ** 2 - 2 * g ** 3, L * (-g ** 2 + g ** 3)])
    Nt = np.array([1 - g, g])
    bend, tors = [0, 1, 3, 4], [2, 5]
    Ke = np.zeros((6, 6))
    Me = np.zeros((6, 6))
    Ke[np.ix_(bend, bend)] += Kb
    Me[np.ix_(bend, bend)] += Mb
    Ke[np.ix_(tors, tors)] += Kt
    Me[np.ix_(tors, tors)] += Mt
    for i, bi in enumerate(bend):
        for j, tj in enumerate(tors):
            v = m * xc * np.sum(w * Nb[i] * Nt[j]) * L
            Me[bi, tj] += v
            Me[tj, bi] += v
    return Ke, Me


class Beam:
    def __init__(self, length, n_elements, EI, GJ, m_per_length, Ip, x_ea_cg=0.0,
                 structural_damping=0.0):
        self.nelem = n_elements
        self.nnodes = n_elements + 1
        self.ndof = 3 * self.nnodes
        self.Le = length / n_elements
        self.y_nodes = np.linspace(0.0, length, self.nnodes)
        self.K = np.zeros((self.ndof, self.ndof))
        self.M = np.zeros((self.ndof, self.ndof))
        Ke, Me = element_matrices(EI, GJ, m_per_length, Ip, x_ea_cg, self.Le)
        for e in range(n_elements):
            dofs = np.arange(3 * e, 3 * e + 6)
            self.K[np.ix_(dofs, dofs)] += Ke
            self.M[np.ix_(dofs, dofs)] += Me
        self.free = np.arange(3, self.ndof)
        self.C = np.zeros_like(self.K)
        if structural_damping > 0:
            ev = eigh(self.K[np.ix_(self.free, self.free)], self.M[np.ix_(self.free, self.free)],
                      eigvals_only=True)
            self.C = 2 * structural_damping / np.sqrt(max(ev[0], 1e-6)) * self.K
        self.d = np.zeros(self.ndof)
        self.v = np.zeros(self.ndof)
        self.a = np.zeros(self.ndof)

    def frequencies(self):
        ev = eigh(self.K[np.ix_(self.free, self.free)], self.M[np.ix_(self.free, self.free)],
                  eigvals_only=True)
        return np.sqrt(np.maximum(ev, 0.0)) / (2 * np.pi)

    def init_acceleration(self):
        f = self.free
        self.a[f] = np.linalg.solve(self.M[np.ix_(f, f)], -self.K[np.ix_(f, f)] @ self.d[f])

    def step(self, F, dt, beta=0.25, gamma=0.5):
        f = self.free
        K, M, C = (X[np.ix_(f, f)] for X in (self.K, self.M, self.C))
        d, v, a = self.d[f], self.v[f], self.a[f]
        Keff = K + gamma / (beta * dt) * C + 1 / (beta * dt ** 2) * M
        Feff = (F[f] + M @ (d / (beta * dt ** 2) + v / (beta * dt) + (1 / (2 * beta) - 1) * a)
                + C @ (gamma / (beta * dt) * d + (gamma / beta - 1) * v
                       + dt * (gamma / (2 * beta) - 1) * a))
        dn = np.linalg.solve(Keff, Feff)
        an = (dn - d) / (beta * dt ** 2) - v / (beta * dt) - (1 / (2 * beta) - 1) * a
        vn = v + dt * ((1 - gamma) * a + gamma * an)
        self.d[:] = 0.0
        self.v[:] = 0.0
        self.a[:] = 0.0
        self.d[f], self.v[f], self.a[f] = dn, vn, an


def distribute(y_nodes, y_f, lift, moment=None):
    """Station forces (and moments) to nodal [w, dw/dy, theta] loads by linear
    interpolation between the bracketing nodes."""
    N = len(y_nodes)
    F = np.zeros(3 * N)
    for k in range(len(y_f)):
        idx = int(np.searchsorted(y_nodes, y_f[k], side="right") - 1)
        idx = max(0, min(idx, N - 2))
        xi = (y_f[k] - y_nodes[idx]) / (y_nodes[idx + 1] - y_nodes[idx])
        xi = max(0.0, min(xi, 1.0))
        F[3 * idx] += lift[k] * (1 - xi)
        F[3 * (idx + 1)] += lift[k] * xi
        if moment is not None:
            F[3 * idx + 2] += moment[k] * (1 - xi)
            F[3 * (idx + 1) + 2] += moment[k] * xi
    return F
