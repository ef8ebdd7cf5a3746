"""Euler-Bernoulli beam FE of the flutter sweep (mirror of src/fluxvortex/beam_fe.py).

Cantilevered wing beam with coupled bending and torsion: 3 DOF per node
[w, dw/dy, theta], Hermite cubic bending and linear torsion elements, the
bending-torsion mass coupling of a CG offset from the elastic axis,
stiffness-proportional Rayleigh damping C = (2 zeta / omega_1) K, and
Newmark average-acceleration stepping (beam_fe.py:27-351 of the reference).

The matrices are assembled once on the host (FP64).  The time step runs on
the device inside the flutter-sweep kernel; because dt is fixed per sweep,
the effective stiffness K_eff = K + gamma/(beta dt) C + 1/(beta dt^2) M of
the root-clamped system is factored once here and the device applies its
inverse (a 24 x 24 FP64 matrix for 8 elements) every step.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

NEWMARK_BETA, NEWMARK_GAMMA = 0.25, 0.5


def _element(EI, GJ, m, Ip, xc, L):
    """6 x 6 element stiffness and mass, DOF [w1, w1', t1, w2, w2', t2]."""
    K = np.zeros((6, 6))
    M = np.zeros((6, 6))
    b = np.array([0, 1, 3, 4])
    t = np.array([2, 5])
    K[np.ix_(b, b)] = EI / L ** 3 * np.array(
        [[12, 6 * L, -12, 6 * L], [6 * L, 4 * L * L, -6 * L, 2 * L * L],
         [-12, -6 * L, 12, -6 * L], [6 * L, 2 * L * L, -6 * L, 4 * L * L]])
    M[np.ix_(b, b)] = m * L / 420 * np.array(
        [[156, 22 * L, 54, -13 * L], [22 * L, 4 * L * L, 13 * L, -3 * L * L],
         [54, 13 * L, 156, -22 * L], [-13 * L, -3 * L * L, -22 * L, 4 * L * L]])
    K[np.ix_(t, t)] = GJ / L * np.array([[1.0, -1.0], [-1.0, 1.0]])
    M[np.ix_(t, t)] = Ip * L / 6 * np.array([[2.0, 1.0], [1.0, 2.0]])
    # coupling m x_c int N_bend N_tors dy: 3-point Gauss on [0, 1] (exact: degree 4)
    q = 0.5 + 0.5 * np.sqrt(0.6) * np.array([-1.0, 0.0, 1.0])
    wq = np.array([5.0, 8.0, 5.0]) / 18.0
    nb = np.stack([1 - 3 * q * q + 2 * q ** 3, L * (q - 2 * q * q + q ** 3), 3 * q * q - 2 * q ** 3,
                   L * (q ** 3 - q * q)])
    nt = np.stack([1 - q, q])
    Mc = m * xc * L * (nb * wq) @ nt.T        # (4, 2)
    M[np.ix_(b, t)] += Mc
    M[np.ix_(t, b)] += Mc.T
    return K, M


@dataclass
class BeamModel:
    length: float
    n_elements: int
    EI: float
    GJ: float
    m_per_length: float
    Ip: float
    x_ea_cg: float = 0.0
    structural_damping: float = 0.0

    def __post_init__(self):
        n = self.n_elements
        self.nnodes = n + 1
        self.ndof = 3 * self.nnodes
        self.y_nodes = np.linspace(0.0, self.length, self.nnodes)
        Ke, Me = _element(self.EI, self.GJ, self.m_per_length, self.Ip, self.x_ea_cg,
                          self.length / n)
        self.K = np.zeros((self.ndof, self.ndof))
        self.M = np.zeros((self.ndof, self.ndof))
        for e in range(n):
            s = slice(3 * e, 3 * e + 6)
            self.K[s, s] += Ke
            self.M[s, s] += Me
        self.free = np.arange(3, self.ndof)        # root node clamped
        f = self.free
        self.Kr = self.K[np.ix_(f, f)]
        self.Mr = self.M[np.ix_(f, f)]
        self.Cr = np.zeros_like(self.Kr)
        if self.structural_damping > 0:
            w1 = np.sqrt(max(self.eigenvalues()[0], 1e-6))
            self.Cr = 2.0 * self.structural_damping / w1 * self.Kr

    def eigenvalues(self):
        # generalised symmetric eigenproblem through the Cholesky factor of M
        Lc = np.linalg.cholesky(self.Mr)
        Li = np.linalg.inv(Lc)
        return np.linalg.eigvalsh(Li @ self.Kr @ Li.T)

    def frequencies(self):
        return np.sqrt(np.maximum(self.eigenvalues(), 0.0)) / (2.0 * np.pi)

    def newmark_inverse(self, dt):
        """Inverse of the reduced effective stiffness for step dt."""
        b, g = NEWMARK_BETA, NEWMARK_GAMMA
        Keff = self.Kr + g / (b * dt) * self.Cr + 1.0 / (b * dt * dt) * self.Mr
        return np.linalg.inv(Keff)

    def initial_state(self, tip_w=0.0, tip_theta=0.0):
        """(d, v, a) over all DOF with a tip perturbation and a = M^-1 (-K d)."""
        d = np.zeros(self.ndof)
        d[3 * (self.nnodes - 1)] = tip_w
        d[3 * (self.nnodes - 1) + 2] = tip_theta
        a = np.zeros(self.ndof)
        a[self.free] = np.linalg.solve(self.Mr, -self.Kr @ d[self.free])
        return d, np.zeros(self.ndof), a
