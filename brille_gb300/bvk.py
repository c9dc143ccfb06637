"""Synthetic Born–von Kármán lattice dynamics: the exact model that fills
trellis vertices and scores interpolation error.

Central pair springs k(r) = exp(-r / decay) eV/Å² between every pair of atoms
closer than `cutoff`, force constants Φ_kk'(L) = −k r̂ r̂ᵀ, the self term fixed
by the acoustic sum rule.  The dynamical matrix carries the phase of the cell
translation only,

    D_{kα,k'β}(q) = Σ_L Φ_{kα,k'β}(L) exp(2πi q·n_L) / √(m_k m_k'),

which is the eigenvector convention the Γ rotation of the query path assumes.
Eigenvalues are returned as ħω in meV (negative for unstable modes),
eigenvectors as (modes, atoms, 3) complex Cartesian components.

The reference has no such generator; this model is checked by its own tests
(Hermiticity, acoustic sum rule at Γ, ω(Rq) = ω(q), eigenvectors related by
the Γ table).
"""
from __future__ import annotations

import itertools

import numpy as np

from .crystal import Lattice

# sqrt(eV / (Å² amu)) in rad/s times ħ in meV·s
HBAR_OMEGA_MEV = 64.65415129


class BvKModel:
    def __init__(self, lattice: Lattice, masses, cutoff=6.0, decay=1.5):
        self.lattice = lattice
        self.masses = np.asarray(masses, float).ravel()
        pos = lattice.basis.positions
        n = pos.shape[0]
        if self.masses.size != n:
            raise ValueError("one mass per basis atom is required")
        A = lattice.A
        reach = int(np.ceil(cutoff / np.min(np.linalg.norm(A, axis=1)))) + 1
        cells = np.array(list(itertools.product(range(-reach, reach + 1), repeat=3)))
        terms = []  # (k, k', n_L, Φ 3×3)
        self_term = np.zeros((n, 3, 3))
        for k in range(n):
            for kp in range(n):
                d = (pos[kp][None, :] + cells - pos[k][None, :]) @ A
                r = np.linalg.norm(d, axis=1)
                for c in np.nonzero((r <= cutoff) & (r > 1e-8))[0]:
                    rh = d[c] / r[c]
                    phi = -np.exp(-r[c] / decay) * np.outer(rh, rh)
                    terms.append((k, kp, cells[c], phi))
                    self_term[k] -= phi
        self.n_atoms = n
        self.n_modes = 3 * n
        ks = np.array([t[0] for t in terms], int)
        kps = np.array([t[1] for t in terms], int)
        self._k, self._kp = ks, kps
        self._nL = np.array([t[2] for t in terms], float)
        self._phi = np.array([t[3] for t in terms])
        self._self = self_term
        self._inv_sqrt_m = 1.0 / np.sqrt(self.masses)

    def dynamical_matrix(self, q_rlu):
        """(N, 3n, 3n) Hermitian dynamical matrices at conventional r.l.u. q."""
        q = np.atleast_2d(np.asarray(q_rlu, float))
        N, n = q.shape[0], self.n_atoms
        D = np.zeros((N, n, 3, n, 3), complex)
        ph = np.exp(2j * np.pi * (q @ self._nL.T))  # (N, T)
        for t in range(len(self._k)):
            D[:, self._k[t], :, self._kp[t], :] += ph[:, t, None, None] * self._phi[t][None]
        for k in range(n):
            D[:, k, :, k, :] += self._self[k][None]
        s = self._inv_sqrt_m
        D *= s[None, :, None, None, None] * s[None, None, None, :, None]
        return D.reshape(N, 3 * n, 3 * n)

    def modes(self, q_rlu, chunk=4096):
        """(ħω meV (N, 3n), eigenvectors (N, 3n, n, 3)) sorted by energy."""
        q = np.atleast_2d(np.asarray(q_rlu, float))
        N, n = q.shape[0], self.n_atoms
        w = np.empty((N, 3 * n))
        v = np.empty((N, 3 * n, n, 3), complex)
        for a in range(0, N, chunk):
            D = self.dynamical_matrix(q[a:a + chunk])
            D = 0.5 * (D + np.conj(np.swapaxes(D, 1, 2)))
            lam, vec = np.linalg.eigh(D)
            w[a:a + chunk] = np.sign(lam) * np.sqrt(np.abs(lam)) * HBAR_OMEGA_MEV
            v[a:a + chunk] = np.swapaxes(vec, 1, 2).reshape(-1, 3 * n, n, 3)
        return w, v

    def modes_torch(self, q_rlu, device="cuda", chunk=65536):
        """The same on a GPU through torch (FP64 eigh), for large vertex sets."""
        import torch

        q = torch.as_tensor(np.atleast_2d(q_rlu), dtype=torch.float64, device=device)
        nL = torch.as_tensor(self._nL, dtype=torch.float64, device=device)
        phi = torch.as_tensor(self._phi, dtype=torch.complex128, device=device)
        n = self.n_atoms
        k = torch.as_tensor(self._k, device=device)
        kp = torch.as_tensor(self._kp, device=device)
        selfm = torch.as_tensor(self._self, dtype=torch.complex128, device=device)
        s = torch.as_tensor(self._inv_sqrt_m, dtype=torch.float64, device=device)
        scale = (s[:, None, None, None] * s[None, None, :, None]).to(torch.complex128)
        idx = (k * n + kp)
        ws, vs = [], []
        for a in range(0, q.shape[0], chunk):
            qa = q[a:a + chunk]
            ph = torch.exp(2j * np.pi * (qa @ nL.T))                       # (M, T)
            contrib = ph[:, :, None, None] * phi[None]                      # (M, T, 3, 3)
            D = torch.zeros(qa.shape[0], n * n, 3, 3, dtype=torch.complex128, device=device)
            D.index_add_(1, idx, contrib)
            D = D.reshape(-1, n, n, 3, 3)
            ar = torch.arange(n, device=device)
            D[:, ar, ar] += selfm[None]
            D = D.permute(0, 1, 3, 2, 4) * scale[None]
            D = D.reshape(-1, 3 * n, 3 * n)
            D = 0.5 * (D + D.conj().transpose(1, 2))
            lam, vec = torch.linalg.eigh(D)
            ws.append((torch.sign(lam) * torch.sqrt(lam.abs()) * HBAR_OMEGA_MEV).cpu().numpy())
            vs.append(vec.transpose(1, 2).reshape(-1, 3 * n, n, 3).cpu().numpy())
        return np.concatenate(ws), np.concatenate(vs)
