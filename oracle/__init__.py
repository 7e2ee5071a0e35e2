"""ctypes front end of the CPU oracle (oracle/oracle.c).

Test infrastructure only: tests/, __graft_entry__.smoke() and the CPU legs of
bench.py use it to verify results or as the timed CPU baseline.  The GPU
product (manybody_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_i64p = C.POINTER(C.c_int64)
_u64p = C.POINTER(C.c_uint64)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build() -> str:
    """Compile oracle/liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "oracle.c")
        ):
            build()
        L = C.CDLL(_LIB_PATH)
        L.or_basis_size.restype = C.c_int64
        L.or_basis_size.argtypes = [C.c_int, C.c_int, C.c_int]
        L.or_basis_enumerate.restype = C.c_int64
        L.or_basis_enumerate.argtypes = [C.c_int, C.c_int, C.c_int, _u64p, _u64p]
        L.or_hubbard_term_count.restype = C.c_int
        L.or_hubbard_term_count.argtypes = [_ip, C.c_int, C.c_double, C.c_double]
        L.or_matrix_elements_csc.restype = C.c_int64
        L.or_matrix_elements_csc.argtypes = [_ip, C.c_int, C.c_double, C.c_double, C.c_int,
                                             C.c_int, _i64p, _i64p, _dp, _dp, C.c_int64]
        L.or_csc_apply.restype = None
        L.or_csc_apply.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp, _dp]
        L.or_csc_apply_hermitian_parallel.restype = None
        L.or_csc_apply_hermitian_parallel.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp, _dp]
        L.or_max_threads.restype = C.c_int
        L.or_max_threads.argtypes = []
        L.or_philox_uniform_pm1.restype = None
        L.or_philox_uniform_pm1.argtypes = [C.c_uint64, C.c_uint32, C.c_int64, _dp]
        L.or_philox_phase.restype = None
        L.or_philox_phase.argtypes = [C.c_uint64, C.c_uint32, C.c_int64, _dp]
        L.or_tridiag_eig.restype = C.c_int
        L.or_tridiag_eig.argtypes = [C.c_int, _dp, _dp, _dp]
        L.or_find_min_eigenpair.restype = C.c_int
        L.or_find_min_eigenpair.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp, C.c_int,
                                            C.c_int, _dp, _dp, _dp, _dp]
        L.or_time_evolve.restype = C.c_int
        L.or_time_evolve.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp, C.c_double, C.c_int,
                                     C.c_int, _dp]
        L.or_expm_tridiag_first_column.restype = C.c_int
        L.or_expm_tridiag_first_column.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_int, _dp,
                                                   _dp]
        L.or_jackson_kernel.restype = None
        L.or_jackson_kernel.argtypes = [C.c_int, _dp]
        L.or_lorentz_kernel.restype = None
        L.or_lorentz_kernel.argtypes = [C.c_int, C.c_double, _dp]
        L.or_projector_moments.restype = None
        L.or_projector_moments.argtypes = [C.c_int, C.c_double, _dp]
        L.or_kpm_dos_moments.restype = C.c_int
        L.or_kpm_dos_moments.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp, C.c_int,
                                         C.c_double, C.c_double, _dp]
        L.or_kpm_projector_apply.restype = C.c_int
        L.or_kpm_projector_apply.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, C.c_int,
                                             C.c_double, C.c_double, C.c_double, C.c_double,
                                             _dp, _dp]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def basis(L: int, nup: int, ndn: int):
    """Reference-order basis as (up_masks, down_masks) uint64 arrays."""
    n = lib().or_basis_size(L, nup, ndn)
    up = np.zeros(max(n, 1), np.uint64)
    dn = np.zeros(max(n, 1), np.uint64)
    got = lib().or_basis_enumerate(L, nup, ndn, _p(up, _u64p), _p(dn, _u64p))
    assert got == n, (got, n)
    return up[:n], dn[:n]


def term_count(dims, t=1.0, U=2.0) -> int:
    d = np.asarray(dims, np.int32)
    return lib().or_hubbard_term_count(_p(d, _ip), len(dims), t, U)


class CscMatrix:
    """Sparse H as compute_matrix_elements builds it: CSC of H (== CSR of H^T = H)."""

    def __init__(self, dim, col_ptr, row_idx, re, im):
        self.dim = dim
        self.col_ptr, self.row_idx, self.re, self.im = col_ptr, row_idx, re, im

    @property
    def nnz(self):
        return int(self.col_ptr[-1])

    def _args(self):
        return (self.dim, _p(self.col_ptr, _i64p), _p(self.row_idx, _i64p), _p(self.re, _dp),
                _p(self.im, _dp))

    def apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.complex128)
        y = np.empty(self.dim, np.complex128)
        lib().or_csc_apply(*self._args(), _p(x.view(np.float64), _dp), _p(y.view(np.float64), _dp))
        return y

    def apply_parallel(self, x: np.ndarray) -> np.ndarray:
        """Multi-core row gather for Hermitian H (column i is the conjugate of
        row i): best-effort CPU context, not the reference's serial scatter."""
        x = np.ascontiguousarray(x, np.complex128)
        y = np.empty(self.dim, np.complex128)
        lib().or_csc_apply_hermitian_parallel(*self._args(), _p(x.view(np.float64), _dp),
                                              _p(y.view(np.float64), _dp))
        return y

    def to_dense(self) -> np.ndarray:
        H = np.zeros((self.dim, self.dim), np.complex128)
        for j in range(self.dim):
            s, e = self.col_ptr[j], self.col_ptr[j + 1]
            H[self.row_idx[s:e], j] = self.re[s:e] + 1j * self.im[s:e]
        return H

    def find_min_eigenpair(self, seed_vec, k, reorth=False, want_vec=True):
        seed_vec = np.ascontiguousarray(seed_vec, np.complex128)
        e0 = C.c_double(0.0)
        vec = np.zeros(self.dim, np.complex128) if want_vec else None
        alphas = np.zeros(max(k, 1))
        betas = np.zeros(max(k, 1))
        m = lib().or_find_min_eigenpair(*self._args(), _p(seed_vec.view(np.float64), _dp), k,
                                        int(reorth), C.byref(e0),
                                        _p(vec.view(np.float64), _dp) if want_vec else None,
                                        _p(alphas, _dp), _p(betas, _dp))
        if m < 0:
            raise RuntimeError(f"oracle find_min_eigenpair failed ({m})")
        return e0.value, vec, m, alphas[:m], betas[:max(m - 1, 0)]

    def time_evolve(self, psi0, t, krylov_steps=30, imaginary=False):
        psi0 = np.ascontiguousarray(psi0, np.complex128)
        out = np.zeros(self.dim, np.complex128)
        m = lib().or_time_evolve(*self._args(), _p(psi0.view(np.float64), _dp), t, krylov_steps,
                                 int(imaginary), _p(out.view(np.float64), _dp))
        if m < 0:
            raise RuntimeError("oracle time_evolve failed")
        return out

    def kpm_dos_moments(self, r, M, a, b):
        r = np.ascontiguousarray(r, np.complex128)
        mu = np.zeros(M)
        lib().or_kpm_dos_moments(*self._args(), _p(r.view(np.float64), _dp), M, a, b,
                                 _p(mu, _dp))
        return mu

    def kpm_projector_apply(self, v, M, emin, emax, efermi=0.0, padding=0.01):
        v = np.ascontiguousarray(v, np.complex128)
        out = np.zeros(self.dim, np.complex128)
        lib().or_kpm_projector_apply(*self._args(), M, emin, emax, efermi, padding,
                                     _p(v.view(np.float64), _dp), _p(out.view(np.float64), _dp))
        return out


def hubbard_csc(dims, t, U, nup, ndn) -> CscMatrix:
    """Reference-order H via the restated compute_matrix_elements."""
    d = np.asarray(dims, np.int32)
    L = int(np.prod(dims))
    dim = lib().or_basis_size(L, nup, ndn)
    col_ptr = np.zeros(dim + 1, np.int64)
    nnz = lib().or_matrix_elements_csc(_p(d, _ip), len(dims), t, U, nup, ndn, _p(col_ptr, _i64p),
                                       None, None, None, 0)
    if nnz < 0:
        raise ValueError("oracle: bad Hubbard arguments")
    row_idx = np.zeros(max(nnz, 1), np.int64)
    re = np.zeros(max(nnz, 1))
    im = np.zeros(max(nnz, 1))
    got = lib().or_matrix_elements_csc(_p(d, _ip), len(dims), t, U, nup, ndn, _p(col_ptr, _i64p),
                                       _p(row_idx, _i64p), _p(re, _dp), _p(im, _dp), nnz)
    assert got == nnz
    return CscMatrix(dim, col_ptr, row_idx[:nnz], re[:nnz], im[:nnz])


def max_threads() -> int:
    """OpenMP threads the oracle's parallel loops use."""
    return int(lib().or_max_threads())


def philox_uniform(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """Complex vector with re, im ~ U[-1, 1) from Philox4x32-10, counter = index."""
    out = np.zeros(n, np.complex128)
    lib().or_philox_uniform_pm1(seed, stream, n, _p(out.view(np.float64), _dp))
    return out


def philox_phase(seed: int, n: int, stream: int = 0) -> np.ndarray:
    out = np.zeros(n, np.complex128)
    lib().or_philox_phase(seed, stream, n, _p(out.view(np.float64), _dp))
    return out


def tridiag_eig(alphas, betas):
    n = len(alphas)
    d = np.array(alphas, np.float64)
    e = np.zeros(max(n, 1))
    e[: max(n - 1, 0)] = betas[: max(n - 1, 0)]
    z = np.zeros((n, n), order="F")
    rc = lib().or_tridiag_eig(n, _p(d, _dp), _p(e, _dp), z.ctypes.data_as(_dp))
    if rc:
        raise RuntimeError("tridiagonal eigensolve did not converge")
    return d, z


def jackson_kernel(N):
    g = np.zeros(N + 1)
    lib().or_jackson_kernel(N, _p(g, _dp))
    return g


def lorentz_kernel(N, lam=4.0):
    g = np.zeros(N + 1)
    lib().or_lorentz_kernel(N, lam, _p(g, _dp))
    return g


def projector_moments(M, eps):
    mu = np.zeros(M + 1)
    lib().or_projector_moments(M, eps, _p(mu, _dp))
    return mu


def expm_tridiag_first_column(alphas, betas, t, imaginary=False):
    n = len(alphas)
    a = np.array(alphas, np.float64)
    b = np.zeros(max(n, 1))
    b[: max(n - 1, 0)] = betas[: max(n - 1, 0)]
    yr = np.zeros(max(n, 1))
    yi = np.zeros(max(n, 1))
    rc = lib().or_expm_tridiag_first_column(n, _p(a, _dp), _p(b, _dp), t, int(imaginary),
                                            _p(yr, _dp), _p(yi, _dp))
    if rc:
        raise RuntimeError("expm failed")
    return (yr + 1j * yi)[:n]


def momentum_factorized_matrix(dims, t: float, U: float, up_masks, down_masks) -> np.ndarray:
    """Dense H of the reference's HubbardMomentumFactorized
    (src/numerics/hubbard_momentum_factorized.h:32-249) on the given basis
    (occupation masks over momentum orbitals, reference order):
    H = t diag(sum_k eps(k) n_k) + (U/N) sum_q rho_{q,up} rho_{-q,down}, with
    eps(k) = -2 sum_d cos(2 pi k_d / L_d) (:107-133) and rho_{q,s} =
    sum_k c+_{k+q,s} c_{k,s} built per column as :136-237 does: the key lists
    the up creators then the down creators, each by ascending orbital; moving
    k -> k+q costs (-1)^(op_idx + insert_pos).  Flat momentum index: first
    dimension fastest (src/utils/index.h).  Pure Python, small bases only."""
    dims = [int(d) for d in dims]
    N = int(np.prod(dims))
    strides = np.cumprod([1] + dims[:-1])

    def coords(k):
        return [(k // strides[d]) % dims[d] for d in range(len(dims))]

    def flat(c):
        return int(sum(c[d] * strides[d] for d in range(len(dims))))

    def add(k, q, sign):
        a, b = coords(k), coords(q)
        return flat([(a[d] + sign * b[d]) % dims[d] for d in range(len(dims))])

    eps = [-2.0 * sum(np.cos(2.0 * np.pi * c / dims[d]) for d, c in enumerate(coords(k)))
           for k in range(N)]
    keys = list(zip((int(u) for u in up_masks), (int(d) for d in down_masks)))
    index = {k: i for i, k in enumerate(keys)}
    n = len(keys)

    def rho(q, spin):
        R = np.zeros((n, n))
        for j, (um, dm) in enumerate(keys):
            mine = um if spin == 0 else dm
            orbs = [o for o in range(N) if (mine >> o) & 1]
            before = 0 if spin == 0 else bin(um).count("1")  # up creators precede down ones
            for pos, k in enumerate(orbs):
                kq = add(k, q, +1)
                if kq == k:
                    R[j, j] += 1.0
                    continue
                if (mine >> kq) & 1:
                    continue
                rest = mine & ~(1 << k)
                insert = before + bin(rest & ((1 << kq) - 1)).count("1")
                sign = -1.0 if (before + pos + insert) % 2 else 1.0
                new = rest | (1 << kq)
                key = (new, dm) if spin == 0 else (um, new)
                if key in index:
                    R[index[key], j] += sign
        return R

    H = np.diag([t * sum(eps[o] for o in range(N) if (um >> o) & 1) +
                 t * sum(eps[o] for o in range(N) if (dm >> o) & 1) for um, dm in keys])
    if abs(U) > 1e-15:
        for q in range(N):
            H = H + (U / N) * (rho(q, 0) @ rho(add(0, q, -1), 1))
    return H
