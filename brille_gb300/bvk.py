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

import contextlib
import itertools
import os

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
        # mass-weighted force constants summed per cell translation:
        # D(q) = Σ_L exp(2πi q·n_L) Ψ_L, Ψ_L a (3n × 3n) matrix
        cells_used, inv = np.unique(self._nL, axis=0, return_inverse=True)
        psi = np.zeros((len(cells_used), n, 3, n, 3))
        for t in range(len(ks)):
            psi[inv[t], ks[t], :, kps[t], :] += self._phi[t]
        zero = np.nonzero(np.all(cells_used == 0, axis=1))[0]
        if len(zero) == 0:
            cells_used = np.vstack([cells_used, np.zeros(3)])
            psi = np.concatenate([psi, np.zeros((1, n, 3, n, 3))])
            zero = [len(cells_used) - 1]
        for k in range(n):
            psi[zero[0], k, :, k, :] += self_term[k]
        sm = self._inv_sqrt_m
        psi *= sm[None, :, None, None, None] * sm[None, None, None, :, None]
        self._cells = cells_used
        self._psi = psi.reshape(len(cells_used), 9 * n * n)

    def dynamical_matrix(self, q_rlu):
        """(N, 3n, 3n) Hermitian dynamical matrices at conventional r.l.u. q."""
        q = np.atleast_2d(np.asarray(q_rlu, float))
        ph = np.exp(2j * np.pi * (q @ self._cells.T))  # (N, cells)
        D = ph @ self._psi
        return D.reshape(len(q), 3 * self.n_atoms, 3 * self.n_atoms)

    def _modes_serial(self, q):
        n = self.n_atoms
        D = self.dynamical_matrix(q)
        D = 0.5 * (D + np.conj(np.swapaxes(D, 1, 2)))
        lam, vec = np.linalg.eigh(D)
        w = np.sign(lam) * np.sqrt(np.abs(lam)) * HBAR_OMEGA_MEV
        v = np.swapaxes(vec, 1, 2).reshape(-1, 3 * n, n, 3)
        return w, v

    def modes(self, q_rlu, chunk=4096, processes=0):
        """(ħω meV (N, 3n), eigenvectors (N, 3n, n, 3)) sorted by energy.

        processes > 1 spreads the eigensolves over a spawn-started process
        pool (safe in a process that has already initialised CUDA; the caller's
        __main__ must be importable, i.e. a file, not standard input)."""
        q = np.atleast_2d(np.asarray(q_rlu, float))
        N, n = q.shape[0], self.n_atoms
        w = np.empty((N, 3 * n))
        v = np.empty((N, 3 * n, n, 3), complex)
        parts = [(a, min(N, a + chunk)) for a in range(0, N, chunk)]
        if processes > 1 and len(parts) > 1:
            from multiprocessing import shared_memory

            shm_w = shared_memory.SharedMemory(create=True, size=w.nbytes)
            shm_v = shared_memory.SharedMemory(create=True, size=v.nbytes)
            try:
                _run_pool(processes, _modes_worker, [(self, q[a:b], a, N, shm_w.name, shm_v.name) for a, b in parts])
                w[:] = np.ndarray(w.shape, w.dtype, buffer=shm_w.buf)
                v[:] = np.ndarray(v.shape, v.dtype, buffer=shm_v.buf)
            finally:
                for s_ in (shm_w, shm_v):
                    s_.close()
                    s_.unlink()
        else:
            for a, b in parts:
                w[a:b], v[a:b] = self._modes_serial(q[a:b])
        return w, v

    def frequencies(self, q_rlu, chunk=8192, processes=0):
        """ħω in meV (N, 3n), sorted, without eigenvectors (eigvalsh)."""
        q = np.atleast_2d(np.asarray(q_rlu, float))
        N = q.shape[0]
        w = np.empty((N, self.n_modes))
        parts = [(a, min(N, a + chunk)) for a in range(0, N, chunk)]
        if processes > 1 and len(parts) > 1:
            from multiprocessing import shared_memory

            shm = shared_memory.SharedMemory(create=True, size=w.nbytes)
            try:
                _run_pool(processes, _freq_worker, [(self, q[a:b], a, N, shm.name) for a, b in parts])
                w[:] = np.ndarray(w.shape, w.dtype, buffer=shm.buf)
            finally:
                shm.close()
                shm.unlink()
        else:
            for a, b in parts:
                w[a:b] = self._freq_serial(q[a:b])
        return w

    def _freq_serial(self, q):
        D = self.dynamical_matrix(q)
        D = 0.5 * (D + np.conj(np.swapaxes(D, 1, 2)))
        lam = np.linalg.eigvalsh(D)
        return np.sign(lam) * np.sqrt(np.abs(lam)) * HBAR_OMEGA_MEV


# BLAS thread counts the pool's workers start with: one each, since the
# pool already has one worker per core (16 workers with 16 BLAS threads each
# run the small batched eigensolves several times slower than 16 with one)
_WORKER_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


@contextlib.contextmanager
def spawn_pool(processes):
    """A spawn-started process pool whose workers run single-threaded BLAS
    (safe in a process that has already initialised CUDA).  The variables
    are set while the pool lives, because workers start on first use."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    saved = {k: os.environ.get(k) for k in _WORKER_THREAD_VARS}
    os.environ.update({k: "1" for k in _WORKER_THREAD_VARS})
    try:
        with ProcessPoolExecutor(max_workers=processes, mp_context=mp.get_context("spawn")) as ex:
            yield ex
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def modes_each(items, on_item, processes=0, chunk=4096):
    """modes() of many (model, q_rlu) items through one process pool, one
    item at a time: on_item(i, w, v) receives each item's results before the
    next item starts, so only one item's eigenvectors are held at once."""
    from multiprocessing import shared_memory

    if processes <= 1:
        for i, (model, q) in enumerate(items):
            on_item(i, *model.modes(q, chunk=chunk))
        return
    with spawn_pool(processes) as ex:
        for i, (model, q) in enumerate(items):
            q = np.atleast_2d(np.asarray(q, float))
            N, n = q.shape[0], model.n_atoms
            shm_w = shared_memory.SharedMemory(create=True, size=max(1, N * 3 * n * 8))
            shm_v = shared_memory.SharedMemory(create=True, size=max(1, N * 3 * n * n * 3 * 16))
            try:
                # at least two parts per worker where the item allows
                step = max(64, min(chunk, -(-N // (2 * processes))))
                parts = [(a, min(N, a + step)) for a in range(0, N, step)]
                for f in [ex.submit(_modes_worker, model, q[a:b], a, N, shm_w.name, shm_v.name) for a, b in parts]:
                    f.result()
                on_item(i, np.ndarray((N, 3 * n), float, buffer=shm_w.buf),
                        np.ndarray((N, 3 * n, n, 3), complex, buffer=shm_v.buf))
            finally:
                for s_ in (shm_w, shm_v):
                    s_.close()
                    s_.unlink()


def _run_pool(processes, fn, jobs):
    """Run fn(*job) for every job on a spawn-started process pool.  A worker
    that cannot start (e.g. a __main__ that spawn cannot re-import) raises
    BrokenProcessPool here instead of being restarted forever."""
    with spawn_pool(processes) as ex:
        for f in [ex.submit(fn, *j) for j in jobs]:
            f.result()


def _freq_worker(model, q, a, N, name):
    from multiprocessing import shared_memory

    wa = model._freq_serial(q)
    s = shared_memory.SharedMemory(name=name)
    try:
        np.ndarray((N, model.n_modes), float, buffer=s.buf)[a:a + len(q)] = wa
    finally:
        s.close()


def _modes_worker(model, q, a, N, name_w, name_v):
    from multiprocessing import shared_memory

    n = model.n_atoms
    wa, va = model._modes_serial(q)
    sw = shared_memory.SharedMemory(name=name_w)
    sv = shared_memory.SharedMemory(name=name_v)
    try:
        np.ndarray((N, 3 * n), float, buffer=sw.buf)[a:a + len(q)] = wa
        np.ndarray((N, 3 * n, n, 3), complex, buffer=sv.buf)[a:a + len(q)] = va
    finally:
        sw.close()
        sv.close()
