"""manybody_gb300 -- GB300 matrix-free Hubbard engine, Python front end.

Mirrors the calling surface of keyehzy/manybody's hot path
(FermionBasis / HubbardModel{,2D,3D} / compute_matrix_elements /
LinearOperator + Lanczos, KPM and Krylov evolution) over the C ABI in
include/manybody_gb300.h, implemented by the in-tree CUDA library
manybody_gb300/libmanybody_gb300.so (built by manybody_gb300/build.py).

Device vectors are torch CUDA tensors of dtype complex128 (MB_PREC_F64) or
complex64 (MB_PREC_F32); torch supplies allocation and streams only.  There
is no CPU fallback: without the native library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmanybody_gb300.so")

MB_OK = 0
MB_ERR_INVALID_ARG = 1
MB_ERR_CAPACITY = 2
MB_ERR_ZERO_NORM = 3
MB_ERR_DIM_MISMATCH = 4
MB_ERR_EIG_FAILED = 5
MB_ERR_OOM = 6
MB_ERR_TIMEOUT = 7
MB_ERR_CUDA = 8
MB_ERR_NO_DEVICE = 9

ORDER_REFERENCE = 0
ORDER_TENSOR = 1

PREC_F64 = 0
PREC_F32 = 1
PREC_Q64 = 2

_STATUS_NAMES = {
    1: "MB_ERR_INVALID_ARG", 2: "MB_ERR_CAPACITY", 3: "MB_ERR_ZERO_NORM",
    4: "MB_ERR_DIM_MISMATCH", 5: "MB_ERR_EIG_FAILED", 6: "MB_ERR_OOM", 7: "MB_ERR_TIMEOUT",
    8: "MB_ERR_CUDA", 9: "MB_ERR_NO_DEVICE",
}


class MbError(RuntimeError):
    """A non-zero mb_status from the native library."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None

_i64 = C.c_int64
_i64p = C.POINTER(C.c_int64)
_u64p = C.POINTER(C.c_uint64)
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


class SectorDesc(C.Structure):
    _fields_ = [("dims", C.c_int64 * 3), ("ndim", C.c_int), ("n_up", C.c_int), ("n_down", C.c_int),
                ("t", C.c_double), ("u", C.c_double)]


class LanczosOpts(C.Structure):
    _fields_ = [("reorth", C.c_int), ("basis_precision", C.c_int), ("conv_tol", C.c_double),
                ("check_every", C.c_int), ("refine", C.c_int)]


class EngineShape(C.Structure):
    """mb_engine_shape: the engine step's launch shape."""
    _fields_ = [("persistent", C.c_int), ("row_min_cols", C.c_int), ("ctas_per_sm", C.c_int),
                ("grid", C.c_int), ("warps", C.c_int), ("reserved", C.c_int * 3)]


class ApplyShape(C.Structure):
    """mb_apply_shape: how a lattice operator's H|psi> runs on the GPU."""
    _fields_ = [("passes", C.c_int), ("row_split", C.c_int), ("table_bits", C.c_int),
                ("prefetch", C.c_int), ("table_stage", C.c_int), ("csr_lanes", C.c_int),
                ("reserved", C.c_int * 2)]


# name -> (restype, argtypes); every exported symbol of include/manybody_gb300.h.
SIGNATURES = {
    "mb_version": (C.c_int, []),
    "mb_last_error": (C.c_char_p, []),
    "mb_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "mb_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "mb_free": (C.c_int, [_vp]),
    "mb_memcpy": (C.c_int, [_vp, _vp, C.c_size_t, C.c_int]),
    "mb_synchronize": (C.c_int, []),
    "mb_basis_create_fixed_spin": (C.c_int, [_i64, _i64, C.c_int, C.POINTER(_vp)]),
    "mb_basis_destroy": (C.c_int, [_vp]),
    "mb_basis_size": (C.c_int, [_vp, _i64p]),
    "mb_basis_sector": (C.c_int, [_vp, _i64p, _i64p, _i64p, _i64p, _i64p]),
    "mb_basis_export_reference_order": (C.c_int, [_vp, _u64p, _u64p]),
    "mb_basis_index_of": (C.c_int, [_vp, C.c_uint64, C.c_uint64, _i64p]),
    "mb_basis_permutation": (C.c_int, [_vp, _i64p]),
    "mb_hubbard_create": (C.c_int, [_i64p, C.c_int, C.c_double, C.c_double, C.POINTER(_vp)]),
    "mb_model_destroy": (C.c_int, [_vp]),
    "mb_model_term_count": (C.c_int, [_vp, _i64p]),
    "mb_compute_matrix_elements_csr": (C.c_int, [_vp, _vp, _i64p, _i64p, _i64p, _dp]),
    "mb_op_create": (C.c_int, [_vp, _vp, C.c_int, C.POINTER(_vp)]),
    "mb_op_create_csr": (C.c_int, [_i64, _i64p, _i64p, _dp, C.c_int, C.POINTER(_vp)]),
    "mb_basis_create_momentum": (C.c_int, [_i64p, C.c_int, _i64, C.c_int, _i64p, C.POINTER(_vp)]),
    "mb_basis_create_fixed_number": (C.c_int, [_i64, _i64, C.POINTER(_vp)]),
    "mb_current_create": (C.c_int, [_i64p, C.c_int, C.c_double, _i64p, C.c_int, C.POINTER(_vp)]),
    "mb_compute_rectangular_matrix_elements_csr": (C.c_int, [_vp, _vp, _vp, _i64p, _i64p, _i64p, _dp]),
    "mb_rect_op_create": (C.c_int, [_vp, _vp, _vp, C.c_int, C.POINTER(_vp)]),
    "mb_rect_op_destroy": (C.c_int, [_vp]),
    "mb_rect_op_dims": (C.c_int, [_vp, _i64p, _i64p]),
    "mb_rect_op_apply": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "mb_current_correlator": (C.c_int, [_vp, _vp, _vp, _i64, C.c_uint64, C.c_double, C.c_double,
                                        _i64, _i64, _dp]),
    "mb_hubbard_momentum_create": (C.c_int, [_i64p, C.c_int, C.c_double, C.c_double, C.POINTER(_vp)]),
    "mb_cereal_write_csr": (C.c_int, [C.c_char_p, _i64, _i64, _i64p, _i64p, _dp]),
    "mb_cereal_read_csr": (C.c_int, [C.c_char_p, _i64p, _i64p, _i64p, _i64p, _i64p, _dp]),
    "mb_op_destroy": (C.c_int, [_vp]),
    "mb_op_dimension": (C.c_int, [_vp, _i64p]),
    "mb_op_precision": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "mb_op_apply": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "mb_op_apply_affine": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, C.c_double, _vp,
                                     C.c_int, _vp]),
    "mb_op_apply_host": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "mb_op_apply_noalloc": (C.c_int, [_vp, _vp, _vp, _vp]),
    "mb_fill_uniform": (C.c_int, [_vp, C.c_uint64, C.c_uint32, _vp, C.c_int, _vp]),
    "mb_fill_phase": (C.c_int, [_vp, C.c_uint64, C.c_uint32, _vp, C.c_int, _vp]),
    "mb_lanczos_pass_one": (C.c_int, [_vp, _vp, C.c_int, _i64, C.c_double, _dp, _dp, _i64p, _dp]),
    "mb_lanczos_pass_two": (C.c_int, [_vp, _vp, C.c_int, C.c_double, _dp, _dp, _i64, C.c_double,
                                      _dp, _vp]),
    "mb_find_min_eigenpair": (C.c_int, [_vp, _i64, _vp, C.c_int, C.POINTER(LanczosOpts), _dp, _vp,
                                        _i64p]),
    "mb_find_max_eigenpair": (C.c_int, [_vp, _i64, _vp, C.c_int, C.POINTER(LanczosOpts), _dp, _vp,
                                        _i64p]),
    "mb_time_evolve": (C.c_int, [_vp, _vp, C.c_int, C.c_double, _i64, C.c_int, _vp]),
    "mb_time_evolve_steps": (C.c_int, [_vp, _vp, C.c_int, C.c_double, C.c_double, C.c_double,
                                       _i64]),
    "mb_kpm_dos_moments": (C.c_int, [_vp, _i64, _i64, C.c_uint64, C.c_double, C.c_double,
                                     C.c_double, _dp]),
    "mb_kpm_jackson_kernel": (C.c_int, [_i64, _dp]),
    "mb_kpm_lorentz_kernel": (C.c_int, [_i64, C.c_double, _dp]),
    "mb_kpm_projector_apply": (C.c_int, [_vp, _i64, C.c_double, C.c_double, C.c_double,
                                         C.c_double, _vp, C.c_int, _vp]),
    "mb_estimate_bounds": (C.c_int, [_vp, _i64, C.c_double, C.c_uint64, _dp, _dp]),
    "mb_q64_mantissa_bits": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "mb_q64_from_f64": (C.c_int, [_vp, _vp, C.c_int, _vp, C.POINTER(C.c_int), _vp]),
    "mb_q64_to_f64": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _vp, _vp]),
    "mb_op_apply_q64": (C.c_int, [_vp, _vp, C.c_int, _vp, C.POINTER(C.c_int), _vp]),
    "mb_engine_create": (C.c_int, [_i64, C.POINTER(_vp)]),
    "mb_engine_destroy": (C.c_int, [_vp]),
    "mb_engine_footprint": (C.c_int, [C.POINTER(SectorDesc), _i64p]),
    "mb_engine_submit_ground_state": (C.c_int, [_vp, C.POINTER(SectorDesc), C.c_uint64, _i64,
                                                C.c_double, C.c_int, _i64p]),
    "mb_engine_submit_dos": (C.c_int, [_vp, C.POINTER(SectorDesc), _i64, _i64, C.c_uint64,
                                       C.c_double, _i64p]),
    "mb_engine_poll_dos": (C.c_int, [_vp, _i64, C.POINTER(C.c_int), _dp, _dp, _dp, _dp]),
    "mb_engine_step": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "mb_engine_step_fixed": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "mb_engine_poll": (C.c_int, [_vp, _i64, C.POINTER(C.c_int), _dp, _dp, _i64p, _dp]),
    "mb_engine_set_warps": (C.c_int, [_vp, C.c_int]),
    "mb_engine_set_fused_threshold": (C.c_int, [_vp, C.c_int64]),
    "mb_engine_completed": (C.c_int, [_vp, _i64p, C.c_int64, _i64p]),
    "mb_engine_stats": (C.c_int, [_vp, _i64p, _dp, _dp]),
    "mb_engine_autotune": (C.c_int, [_vp, C.POINTER(C.c_int), _dp]),
    "mb_engine_set_persistent": (C.c_int, [_vp, C.c_int]),
    "mb_engine_set_wait_budget": (C.c_int, [_vp, C.c_int64]),
    "mb_engine_set_basis_limit": (C.c_int, [_vp, C.c_int64]),
    "mb_engine_get_shape": (C.c_int, [_vp, C.POINTER(EngineShape)]),
    "mb_engine_set_shape": (C.c_int, [_vp, C.POINTER(EngineShape)]),
    "mb_op_get_apply_shape": (C.c_int, [_vp, C.POINTER(ApplyShape)]),
    "mb_op_set_apply_shape": (C.c_int, [_vp, C.POINTER(ApplyShape)]),
    "mb_op_autotune": (C.c_int, [_vp, _vp, C.POINTER(ApplyShape), _dp]),
    "mb_dot_re": (C.c_int, [_vp, _vp, _vp, _dp]),
    "mb_norm": (C.c_int, [_vp, _vp, _dp]),
}


def lib():
    """The loaded native library; raises if it was never built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"native library missing: {LIB_PATH} (run `python -m manybody_gb300.build`)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != MB_OK:
        raise MbError(status, lib().mb_last_error().decode(errors="replace"))


def device_count() -> int:
    n = C.c_int(0)
    lib().mb_device_count(C.byref(n))
    return n.value


def _ptr(t) -> int:
    """Device pointer of a torch tensor (or an int)."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_contiguous():
        raise ValueError("vectors must be contiguous")
    return t.data_ptr()


# ---------------------------------------------------------------------------
# FermionBasis (src/algebra/fermion/basis.h)
# ---------------------------------------------------------------------------
class FermionBasis:
    """Fixed-(N, Sz) fermion basis; mirrors BasisImpl (src/algebra/basis.h:12-76)."""

    def __init__(self, handle, orbitals, particles):
        self._h = handle
        self.orbitals = orbitals
        self.particles = particles

    @classmethod
    def with_fixed_particle_number_and_spin(cls, orbitals: int, particles: int,
                                            spin_projection: int) -> "FermionBasis":
        h = C.c_void_p()
        _check(lib().mb_basis_create_fixed_spin(orbitals, particles, spin_projection, C.byref(h)))
        return cls(h, orbitals, particles)

    @classmethod
    def with_fixed_particle_number(cls, orbitals: int, particles: int) -> "FermionBasis":
        """with_fixed_particle_number (src/algebra/basis.cpp:69-89): all spin projections."""
        h = C.c_void_p()
        _check(lib().mb_basis_create_fixed_number(orbitals, particles, C.byref(h)))
        return cls(h, orbitals, particles)

    @classmethod
    def with_fixed_particle_number_spin_momentum(cls, orbitals: int, particles: int,
                                                 spin_projection: int, dims,
                                                 momentum) -> "FermionBasis":
        """with_fixed_particle_number_spin_momentum (src/algebra/basis.cpp:128-185):
        the states of total momentum `momentum` on the periodic lattice `dims`."""
        dims = tuple(int(d) for d in dims)
        momentum = tuple(int(k) for k in momentum)
        if int(np.prod(dims)) != orbitals or len(momentum) != len(dims):
            raise ValueError("orbitals must equal the lattice size, momentum one entry per dimension")
        d = (C.c_int64 * len(dims))(*dims)
        k = (C.c_int64 * len(dims))(*momentum)
        h = C.c_void_p()
        _check(lib().mb_basis_create_momentum(d, len(dims), particles, spin_projection, k,
                                              C.byref(h)))
        b = cls(h, orbitals, particles)
        b.dims, b.momentum = dims, momentum
        return b

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mb_basis_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def size(self) -> int:
        n = C.c_int64()
        _check(lib().mb_basis_size(self._h, C.byref(n)))
        return n.value

    def __len__(self):
        return self.size()

    def sector(self):
        v = [C.c_int64() for _ in range(5)]
        _check(lib().mb_basis_sector(self._h, *[C.byref(x) for x in v]))
        L, nu, nd, du, dd = (x.value for x in v)
        return dict(orbitals=L, n_up=nu, n_down=nd, dim_up=du, dim_down=dd)

    def keys(self):
        """(up_masks, down_masks) uint64 arrays in reference index order."""
        n = self.size()
        up = np.zeros(n, np.uint64)
        dn = np.zeros(n, np.uint64)
        _check(lib().mb_basis_export_reference_order(self._h, up.ctypes.data_as(_u64p),
                                                     dn.ctypes.data_as(_u64p)))
        return up, dn

    def index_of(self, up_mask: int, down_mask: int) -> int:
        r = C.c_int64()
        _check(lib().mb_basis_index_of(self._h, up_mask, down_mask, C.byref(r)))
        return r.value

    def contains(self, up_mask: int, down_mask: int) -> bool:
        try:
            self.index_of(up_mask, down_mask)
            return True
        except MbError:
            return False

    def permutation(self) -> np.ndarray:
        """ref_of_tensor[r_up * D_down + r_down] = reference index."""
        p = np.zeros(self.size(), np.int64)
        _check(lib().mb_basis_permutation(self._h, p.ctypes.data_as(_i64p)))
        return p


# ---------------------------------------------------------------------------
# HubbardModel / 2D / 3D (src/algebra/fermion/model/hubbard_model.h)
# ---------------------------------------------------------------------------
class _Hubbard:
    _create = "mb_hubbard_create"

    def __init__(self, t: float, u: float, dims):
        self.t, self.u, self.dims = float(t), float(u), tuple(int(d) for d in dims)
        d = (C.c_int64 * len(self.dims))(*self.dims)
        h = C.c_void_p()
        _check(getattr(lib(), self._create)(d, len(self.dims), self.t, self.u, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mb_model_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def orbitals(self) -> int:
        return int(np.prod(self.dims))

    def term_count(self) -> int:
        """hamiltonian().size(): number of distinct operator terms."""
        n = C.c_int64()
        _check(lib().mb_model_term_count(self._h, C.byref(n)))
        return n.value

    def _part(self, t: float, u: float) -> "_Hubbard":
        m = _Hubbard.__new__(type(self))
        _Hubbard.__init__(m, t, u, self.dims)
        return m

    def kinetic(self) -> "_Hubbard":
        """kinetic() (hubbard_model.h:13-22, :69-84, :141-161): the hopping
        terms alone, as a model (U = 0)."""
        return self._part(self.t, 0.0)

    def interaction(self) -> "_Hubbard":
        """interaction() (hubbard_model.h:24-32, :86-97, :163-176): the
        U n_up n_down terms alone, as a model (t = 0)."""
        return self._part(0.0, self.u)

    def hamiltonian(self) -> "_Hubbard":
        """hamiltonian() = kinetic() + interaction() (hubbard_model.h:34-38)."""
        return self


class HubbardModel(_Hubbard):
    def __init__(self, t, u, size):
        super().__init__(t, u, (size,))


class HubbardModel2D(_Hubbard):
    def __init__(self, t, u, size_x, size_y):
        super().__init__(t, u, (size_x, size_y))


class HubbardModel3D(_Hubbard):
    def __init__(self, t, u, size_x, size_y, size_z):
        super().__init__(t, u, (size_x, size_y, size_z))


class HubbardModelMomentum(_Hubbard):
    """HubbardModelMomentum (src/algebra/fermion/model/hubbard_model_momentum.h:19-180):
    the Hubbard model on momentum orbitals; with a momentum-sector basis it
    gives that sector's H (compute_matrix_elements, GpuHubbardOperator), with
    a whole (N_up, N_down) basis the union of its sectors (the operator of
    HubbardMomentumFactorized)."""
    _create = "mb_hubbard_momentum_create"

    def __init__(self, t, u, size):
        super().__init__(t, u, tuple(size))


@dataclass
class CsrMatrix:
    """Reference-order sparse H: row_ptr (dim+1), col_idx, values (complex128);
    n_cols = 0 means square."""
    dim: int
    row_ptr: np.ndarray
    col_idx: np.ndarray
    values: np.ndarray
    n_cols: int = 0

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    @property
    def cols(self) -> int:
        return self.n_cols or self.dim

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values, self.col_idx, self.row_ptr), shape=(self.dim, self.cols))


class CurrentOperator:
    """HubbardModelMomentum::current(Q, direction)
    (src/algebra/fermion/model/hubbard_model_momentum.h:52-90): J_d(Q), from
    the momentum sector K to K+Q."""

    def __init__(self, t: float, size, transfer, direction: int):
        self.t, self.dims = float(t), tuple(int(d) for d in size)
        self.transfer, self.direction = tuple(int(q) for q in transfer), int(direction)
        d = (C.c_int64 * len(self.dims))(*self.dims)
        q = (C.c_int64 * len(self.dims))(*self.transfer)
        h = C.c_void_p()
        _check(lib().mb_current_create(d, len(self.dims), self.t, q, self.direction, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mb_model_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def term_count(self) -> int:
        n = C.c_int64()
        _check(lib().mb_model_term_count(self._h, C.byref(n)))
        return n.value


def compute_rectangular_matrix_elements(row_basis: FermionBasis, col_basis: FermionBasis,
                                        op: CurrentOperator) -> CsrMatrix:
    """compute_rectangular_matrix_elements (src/algebra/matrix_elements.h:107-167), on GPU."""
    nnz = C.c_int64()
    n = row_basis.size()
    rp = np.zeros(n + 1, np.int64)
    _check(lib().mb_compute_rectangular_matrix_elements_csr(row_basis.handle, col_basis.handle,
                                                            op.handle, C.byref(nnz),
                                                            rp.ctypes.data_as(_i64p), None, None))
    ci = np.zeros(max(nnz.value, 1), np.int64)
    vals = np.zeros(max(nnz.value, 1), np.complex128)
    _check(lib().mb_compute_rectangular_matrix_elements_csr(
        row_basis.handle, col_basis.handle, op.handle, C.byref(nnz), rp.ctypes.data_as(_i64p),
        ci.ctypes.data_as(_i64p), vals.view(np.float64).ctypes.data_as(_dp)))
    k = nnz.value
    return CsrMatrix(n, rp, ci[:k], vals[:k], col_basis.size())


class GpuCurrentOperator:
    """J and J+ between two momentum sectors on the GPU (reference order)."""

    def __init__(self, row_basis: FermionBasis, col_basis: FermionBasis, op: CurrentOperator,
                 precision: int = PREC_F64):
        h = C.c_void_p()
        _check(lib().mb_rect_op_create(row_basis.handle, col_basis.handle, op.handle, precision,
                                       C.byref(h)))
        self._h = h
        self.precision = precision
        self.shape = (row_basis.size(), col_basis.size())

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mb_rect_op_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def apply(self, x, adjoint: bool = False, out=None):
        import torch
        n = self.shape[1] if adjoint else self.shape[0]
        dt = torch.complex64 if self.precision == PREC_F32 else torch.complex128
        y = torch.empty(n, dtype=dt, device="cuda") if out is None else out
        _check(lib().mb_rect_op_apply(self._h, _ptr(x), _ptr(y), int(adjoint),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return y


def current_correlator(op_k: GpuHubbardOperator, op_kq: GpuHubbardOperator,
                       current: GpuCurrentOperator, n_samples: int, seed: int, beta: float,
                       dt: float, steps: int, krylov_steps: int = 30) -> np.ndarray:
    """The optical-conductivity driver's stochastic current-current correlator
    (examples/hubbard_momentum_optical_conductivity.cpp:340-410), on the GPU."""
    _sync_torch()
    c = np.zeros(2 * steps)
    _check(lib().mb_current_correlator(op_k.handle, op_kq.handle, current.handle, n_samples,
                                       seed, beta, dt, steps, krylov_steps,
                                       c.ctypes.data_as(_dp)))
    return c[0::2] + 1j * c[1::2]


def write_cereal(path: str, m: CsrMatrix) -> None:
    """Writes m in the reference's sparse-matrix cache format (cereal binary
    archive of arma::sp_cx_mat, src/utils/arma_cereal.h:9-30)."""
    rp = np.ascontiguousarray(m.row_ptr, np.int64)
    ci = np.ascontiguousarray(m.col_idx, np.int64)
    vals = np.ascontiguousarray(m.values, np.complex128)
    if ci.size == 0:
        ci = np.zeros(1, np.int64)
        vals = np.zeros(1, np.complex128)
    _check(lib().mb_cereal_write_csr(os.fsencode(path), m.dim, m.cols, rp.ctypes.data_as(_i64p),
                                     ci.ctypes.data_as(_i64p), vals.view(np.float64).ctypes.data_as(_dp)))


def read_cereal(path: str) -> CsrMatrix:
    """Reads a matrix in the reference's sparse-matrix cache format."""
    r, c, nz = C.c_int64(), C.c_int64(), C.c_int64()
    _check(lib().mb_cereal_read_csr(os.fsencode(path), C.byref(r), C.byref(c), C.byref(nz), None,
                                    None, None))
    rp = np.zeros(r.value + 1, np.int64)
    ci = np.zeros(max(nz.value, 1), np.int64)
    vals = np.zeros(max(nz.value, 1), np.complex128)
    _check(lib().mb_cereal_read_csr(os.fsencode(path), C.byref(r), C.byref(c), C.byref(nz),
                                    rp.ctypes.data_as(_i64p), ci.ctypes.data_as(_i64p),
                                    vals.view(np.float64).ctypes.data_as(_dp)))
    n = nz.value
    return CsrMatrix(r.value, rp, ci[:n], vals[:n], 0 if c.value == r.value else c.value)


def compute_matrix_elements(basis: FermionBasis, model: _Hubbard) -> CsrMatrix:
    """compute_matrix_elements<sp_cx_mat> (src/algebra/matrix_elements.h:74-105), built on GPU."""
    nnz = C.c_int64()
    dim = basis.size()
    rp = np.zeros(dim + 1, np.int64)
    _check(lib().mb_compute_matrix_elements_csr(basis.handle, model.handle, C.byref(nnz),
                                                rp.ctypes.data_as(_i64p), None, None))
    n = nnz.value
    ci = np.zeros(max(n, 1), np.int64)
    vals = np.zeros(max(n, 1), np.complex128)
    _check(lib().mb_compute_matrix_elements_csr(basis.handle, model.handle, C.byref(nnz),
                                                rp.ctypes.data_as(_i64p), ci.ctypes.data_as(_i64p),
                                                vals.view(np.float64).ctypes.data_as(_dp)))
    return CsrMatrix(dim, rp, ci[:n], vals[:n])


# ---------------------------------------------------------------------------
# Matrix-free operator (replaces SparseComplexMatrixOperator,
# src/numerics/linear_operator.h:81-91) and the Krylov drivers.
# ---------------------------------------------------------------------------
class GpuHubbardOperator:
    """LinearOperator with apply(v) -> H v and dimension(), on the current GPU."""

    def __init__(self, basis: FermionBasis, model: _Hubbard, precision: int = PREC_F64):
        h = C.c_void_p()
        _check(lib().mb_op_create(basis.handle, model.handle, precision, C.byref(h)))
        self._h = h
        self.precision = precision
        self.basis = basis
        self.model = model
        self._dim = basis.size()

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mb_op_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def dimension(self) -> int:
        return self._dim

    @property
    def dtype(self):
        import torch
        return torch.complex64 if self.precision == PREC_F32 else torch.complex128

    def empty(self):
        import torch
        return torch.empty(self._dim, dtype=self.dtype, device="cuda")

    def _v(self, t):
        """Device pointer of a vector of this operator (None passes): a
        contiguous CUDA tensor of its dtype and dimension, else an error
        before the library reads or writes past it."""
        if t is None or isinstance(t, int):
            return _ptr(t)
        if not t.is_cuda or t.dtype != self.dtype or t.numel() != self._dim:
            raise MbError(MB_ERR_INVALID_ARG,
                          f"expected a CUDA {self.dtype} vector of {self._dim} elements, got "
                          f"{t.dtype} {tuple(t.shape)} on {t.device}")
        return _ptr(t)

    def _f64(self, t):
        """Device pointer of a complex128 vector of this operator's dimension."""
        import torch
        if t is None or isinstance(t, int):
            return _ptr(t)
        if not t.is_cuda or t.dtype != torch.complex128 or t.numel() != self._dim:
            raise MbError(MB_ERR_INVALID_ARG,
                          f"expected a CUDA complex128 vector of {self._dim} elements, got "
                          f"{t.dtype} {tuple(t.shape)} on {t.device}")
        return _ptr(t)

    def _q(self, t):
        """Device pointer of a Q64 vector (int64 mantissa pairs) of this operator."""
        import torch
        if t is None or isinstance(t, int):
            return _ptr(t)
        if not t.is_cuda or t.dtype != torch.int64 or t.numel() != 2 * self._dim:
            raise MbError(MB_ERR_INVALID_ARG,
                          f"expected a CUDA int64 ({self._dim}, 2) Q64 vector, got "
                          f"{t.dtype} {tuple(t.shape)} on {t.device}")
        return _ptr(t)

    def _stream(self, stream):
        if stream is None:
            import torch
            return C.c_void_p(torch.cuda.current_stream().cuda_stream)
        return C.c_void_p(int(stream))

    def apply(self, x, out=None, order: int = ORDER_REFERENCE, stream=None):
        """y = H x (LinearOperator::apply, linear_operator.h:41)."""
        y = self.empty() if out is None else out
        _check(lib().mb_op_apply(self._h, self._v(x), self._v(y), order, self._stream(stream)))
        return y

    def apply_affine(self, x, scale=1.0, shift=0.0, beta=0.0, z=None, out=None,
                     order: int = ORDER_REFERENCE, stream=None):
        y = self.empty() if out is None else out
        _check(lib().mb_op_apply_affine(self._h, self._v(x), self._v(y), scale, shift, beta, self._v(z),
                                        order, self._stream(stream)))
        return y

    def apply_noalloc(self, x, out=None, stream=None):
        """Reference-order y = H x that allocates nothing inside the library:
        for callers that own all device memory (see mb_op_apply_noalloc)."""
        y = self.empty() if out is None else out
        _check(lib().mb_op_apply_noalloc(self._h, self._v(x), self._v(y), self._stream(stream)))
        return y

    def apply_host(self, x: np.ndarray, y: np.ndarray, order: int = ORDER_REFERENCE):
        """apply() on host buffers (numpy or pinned torch CPU tensors)."""
        xp = x.ctypes.data if isinstance(x, np.ndarray) else x.data_ptr()
        yp = y.ctypes.data if isinstance(y, np.ndarray) else y.data_ptr()
        _check(lib().mb_op_apply_host(self._h, xp, yp, order))
        return y

    def seed_vector(self, seed: int = 0, stream_id: int = 0, order: int = ORDER_REFERENCE,
                    out=None):
        v = self.empty() if out is None else out
        _check(lib().mb_fill_uniform(self._h, seed, stream_id, self._v(v), order,
                                     self._stream(None)))
        return v

    def phase_vector(self, seed: int, stream_id: int = 0, order: int = ORDER_REFERENCE, out=None):
        v = self.empty() if out is None else out
        _check(lib().mb_fill_phase(self._h, seed, stream_id, self._v(v), order, self._stream(None)))
        return v

    # --- block-floating-point (PREC_Q64) vectors: int64 mantissas + exponent ---
    def q64_empty(self):
        import torch
        return torch.empty((self._dim, 2), dtype=torch.int64, device="cuda")

    def q64_from_f64(self, x, order: int = ORDER_REFERENCE, out=None, stream=None):
        q = self.q64_empty() if out is None else out
        e = C.c_int()
        _check(lib().mb_q64_from_f64(self._h, self._f64(x), order, self._q(q), C.byref(e),
                                     self._stream(stream)))
        return q, e.value

    def q64_to_f64(self, q, exponent: int, order: int = ORDER_REFERENCE, out=None, stream=None):
        y = self.empty() if out is None else out
        _check(lib().mb_q64_to_f64(self._h, self._q(q), exponent, order, self._f64(y),
                                   self._stream(stream)))
        return y

    def apply_q64(self, q, exponent: int, out=None, stream=None):
        """H applied to a Q64 vector (tensor order); returns (mantissas, exponent)."""
        y = self.q64_empty() if out is None else out
        e = C.c_int()
        _check(lib().mb_op_apply_q64(self._h, self._q(q), exponent, self._q(y), C.byref(e),
                                     self._stream(stream)))
        return y, e.value

    def apply_shape(self) -> dict:
        """The kernel shape of this operator's apply (mb_op_get_apply_shape)."""
        sh = ApplyShape()
        _check(lib().mb_op_get_apply_shape(self._h, C.byref(sh)))
        return {"passes": sh.passes, "row_split": sh.row_split, "table_bits": sh.table_bits,
                "prefetch": sh.prefetch, "table_stage": sh.table_stage, "csr_lanes": sh.csr_lanes}

    def set_apply_shape(self, passes: int = 1, row_split: int = 1, table_bits: int = 32,
                        prefetch: int = 0, table_stage: int = 0, csr_lanes: int = 0):
        """Choose the apply's kernel shape (mb_op_set_apply_shape)."""
        sh = ApplyShape()
        sh.passes, sh.row_split, sh.table_bits = passes, row_split, table_bits
        sh.prefetch, sh.table_stage, sh.csr_lanes = prefetch, table_stage, csr_lanes
        _check(lib().mb_op_set_apply_shape(self._h, C.byref(sh)))

    def autotune(self, stream=None):
        """Time every candidate shape on the GPU and keep the fastest
        (mb_op_autotune); returns (shape dict, ms per apply)."""
        sh = ApplyShape()
        ms = C.c_double()
        _check(lib().mb_op_autotune(self._h, self._stream(stream), C.byref(sh), C.byref(ms)))
        return ({"passes": sh.passes, "row_split": sh.row_split, "table_bits": sh.table_bits,
                 "prefetch": sh.prefetch, "table_stage": sh.table_stage,
                 "csr_lanes": sh.csr_lanes}, ms.value)

    def q64_mantissa_bits(self) -> int:
        b = C.c_int()
        _check(lib().mb_q64_mantissa_bits(self._h, C.byref(b)))
        return b.value

    def dot_re(self, x, y) -> float:
        r = C.c_double()
        _check(lib().mb_dot_re(self._h, self._v(x), self._v(y), C.byref(r)))
        return r.value

    def norm(self, x) -> float:
        r = C.c_double()
        _check(lib().mb_norm(self._h, self._v(x), C.byref(r)))
        return r.value


class HubbardMomentumFactorized(GpuHubbardOperator):
    """HubbardMomentumFactorized (src/numerics/hubbard_momentum_factorized.h:32-249):
    H = t sum_k eps(k) n_k + (U/N) sum_q rho_{q,up} rho_{-q,down} on a whole
    (N_up, N_down) basis of momentum orbitals, constructed as the reference's
    (basis, lattice_size, t, U).  On the GPU it is block diagonal over the
    total momentum (one sector operator per K) in the basis's reference order;
    every driver takes it."""

    def __init__(self, basis: FermionBasis, lattice_size, t: float, U: float,
                 precision: int = PREC_F64):
        if not len(lattice_size):
            raise MbError(MB_ERR_INVALID_ARG,
                          "HubbardMomentumFactorized requires at least one dimension")
        self.lattice_size = tuple(int(d) for d in lattice_size)
        super().__init__(basis, HubbardModelMomentum(t, U, self.lattice_size), precision)


class GpuSparseOperator(GpuHubbardOperator):
    """SparseComplexMatrixOperator (src/numerics/linear_operator.h:81-91) on the GPU:
    any square complex sparse matrix (a CsrMatrix, e.g. from read_cereal), with
    the same apply / Krylov / KPM / evolution drivers.  Its index order is the
    matrix's own (reference and tensor order coincide)."""

    def __init__(self, m: CsrMatrix, precision: int = PREC_F64):
        if m.cols != m.dim:
            raise ValueError("a sparse operator needs a square matrix")
        rp = np.ascontiguousarray(m.row_ptr, np.int64)
        ci = np.ascontiguousarray(m.col_idx, np.int64)
        vals = np.ascontiguousarray(m.values, np.complex128)
        if ci.size == 0:
            ci = np.zeros(1, np.int64)
            vals = np.zeros(1, np.complex128)
        h = C.c_void_p()
        _check(lib().mb_op_create_csr(m.dim, rp.ctypes.data_as(_i64p), ci.ctypes.data_as(_i64p),
                                      vals.view(np.float64).ctypes.data_as(_dp), precision,
                                      C.byref(h)))
        self._h = h
        self.precision = precision
        self.basis = None
        self.model = None
        self._dim = m.dim


def _sync_torch():
    import torch
    torch.cuda.synchronize()


@dataclass
class LanczosDecomposition:
    alphas: np.ndarray
    betas: np.ndarray
    steps_taken: int
    b_norm: float


def lanczos_pass_one(op: GpuHubbardOperator, b, k: int, scale: float = 1.0,
                     order: int = ORDER_REFERENCE) -> LanczosDecomposition:
    """lanczos_pass_one (src/numerics/lanczos.h:130-175)."""
    _sync_torch()
    a = np.zeros(max(k, 1))
    bb = np.zeros(max(k, 1))
    steps = C.c_int64()
    bn = C.c_double()
    _check(lib().mb_lanczos_pass_one(op.handle, op._v(b), order, k, scale, a.ctypes.data_as(_dp),
                                     bb.ctypes.data_as(_dp), C.byref(steps), C.byref(bn)))
    m = steps.value
    return LanczosDecomposition(a[:m].copy(), bb[:max(m - 1, 0)].copy(), m, bn.value)


def lanczos_pass_two(op: GpuHubbardOperator, b, decomp: LanczosDecomposition, y_k,
                     scale: float = 1.0, order: int = ORDER_REFERENCE, out=None):
    """lanczos_pass_two (src/numerics/lanczos.h:177-218); y_k complex."""
    _sync_torch()
    x = op.empty() if out is None else out
    y = np.ascontiguousarray(np.asarray(y_k, np.complex128))
    al = np.ascontiguousarray(decomp.alphas, np.float64)
    be = np.ascontiguousarray(decomp.betas if len(decomp.betas) else np.zeros(1), np.float64)
    _check(lib().mb_lanczos_pass_two(op.handle, op._v(b), order, scale, al.ctypes.data_as(_dp),
                                     be.ctypes.data_as(_dp), decomp.steps_taken, decomp.b_norm,
                                     y.view(np.float64).ctypes.data_as(_dp), op._v(x)))
    return x


def solve(op: GpuHubbardOperator, b, k: int, solver, order: int = ORDER_REFERENCE, out=None):
    """solve (src/numerics/lanczos.h:220-237): pass one, y_k = solver(alphas,
    betas) on the host, scaled by |b|, then pass two; zeros if no step ran."""
    decomp = lanczos_pass_one(op, b, k, order=order)
    if decomp.steps_taken == 0:
        x = op.empty() if out is None else out
        x.zero_()
        return x
    y = np.asarray(solver(decomp.alphas, decomp.betas), np.complex128) * decomp.b_norm
    return lanczos_pass_two(op, b, decomp, y, order=order, out=out)


@dataclass
class EigenPair:
    value: float
    vector: object
    steps: int


def _eigenpair(fn, op, k, seed, order, reorth, basis_precision, conv_tol, check_every,
               want_vector, refine=False):
    _sync_torch()
    opts = LanczosOpts(int(reorth), basis_precision, conv_tol, check_every, int(refine))
    e = C.c_double()
    steps = C.c_int64()
    vec = op.empty() if want_vector else None
    _check(fn(op.handle, k, op._v(seed), order, C.byref(opts), C.byref(e), op._v(vec),
              C.byref(steps)))
    return EigenPair(e.value, vec, steps.value)


def find_min_eigenpair(op: GpuHubbardOperator, k: int, seed=None, order: int = ORDER_REFERENCE,
                       reorth: bool = False, basis_precision: int = -1, conv_tol: float = 0.0,
                       check_every: int = 10, want_vector: bool = True,
                       refine: bool = False) -> EigenPair:
    """find_min_eigenpair (src/numerics/lanczos.h:283-290) from a seeded start vector.
    refine (FP32 operators): the energy is the FP64 Rayleigh quotient of the Ritz vector."""
    if seed is None:
        seed = op.seed_vector(0, order=order)
    return _eigenpair(lib().mb_find_min_eigenpair, op, k, seed, order, reorth, basis_precision,
                      conv_tol, check_every, want_vector, refine)


def find_max_eigenpair(op: GpuHubbardOperator, k: int, seed=None, order: int = ORDER_REFERENCE,
                       reorth: bool = False, basis_precision: int = -1, conv_tol: float = 0.0,
                       check_every: int = 10, want_vector: bool = True) -> EigenPair:
    """find_max_eigenpair (src/numerics/lanczos.h:246-281)."""
    if seed is None:
        seed = op.seed_vector(0, order=order)
    return _eigenpair(lib().mb_find_max_eigenpair, op, k, seed, order, reorth, basis_precision,
                      conv_tol, check_every, want_vector)


def time_evolve_state(op: GpuHubbardOperator, psi0, t: float, krylov_steps: int = 30,
                      order: int = ORDER_REFERENCE, out=None):
    """time_evolve_state (src/numerics/evolve_state.h:164-178): exp(-i t H) psi0."""
    _sync_torch()
    y = op.empty() if out is None else out
    _check(lib().mb_time_evolve(op.handle, op._v(psi0), order, t, krylov_steps, 0, op._v(y)))
    return y


def imaginary_time_evolve_state(op: GpuHubbardOperator, psi0, t: float, krylov_steps: int = 30,
                                order: int = ORDER_REFERENCE, out=None):
    """imaginary_time_evolve_state (src/numerics/evolve_state.h): exp(-t H) psi0."""
    _sync_torch()
    y = op.empty() if out is None else out
    _check(lib().mb_time_evolve(op.handle, op._v(psi0), order, t, krylov_steps, 1, op._v(y)))
    return y


def time_evolve_state_steps(op: GpuHubbardOperator, psi, t0: float, t1: float, dt: float,
                            krylov_steps: int = 30, order: int = ORDER_REFERENCE, callback=None):
    """time_evolve_state_steps (src/numerics/evolve_state.h:204-231), in place.
    With a callback(t, psi), it is called at t0 and after every step (steps of
    dt, the last one shortened to end on t1), as the reference does; without
    one the whole loop runs in the library."""
    _sync_torch()
    if callback is None:
        _check(lib().mb_time_evolve_steps(op.handle, op._v(psi), order, t0, t1, dt,
                                          krylov_steps))
        return psi
    if dt == 0.0 or t1 - t0 == 0.0:
        callback(t0, psi)
        return psi
    direction = 1.0 if t1 >= t0 else -1.0
    dt = abs(dt) * direction
    t = t0
    callback(t, psi)
    while (direction > 0 and t < t1) or (direction < 0 and t > t1):
        step = min(dt, t1 - t) if direction > 0 else max(dt, t1 - t)
        psi.copy_(time_evolve_state(op, psi, step, krylov_steps, order))
        t += step
        callback(t, psi)
    return psi


@dataclass
class Rescaling:
    """rescaling::Rescaling (src/numerics/rescaling.h:9-18): H_scaled = (H - b) / a."""
    a: float
    b: float

    def rescale(self, e: float) -> float:
        return (e - self.b) / self.a

    def inverse(self, e_scaled: float) -> float:
        return e_scaled * self.a + self.b


def rescaling_from_bounds(e_min: float, e_max: float, padding: float = 0.01) -> Rescaling:
    """rescaling::from_bounds (src/numerics/rescaling.h:33-38), the KPM drivers' map."""
    return Rescaling((e_max - e_min) / 2.0 * (1.0 + padding), (e_max + e_min) / 2.0)


def kpm_dos_moments(op: GpuHubbardOperator, n_moments: int, n_probes: int, seed: int,
                    e_min: float, e_max: float, padding: float = 0.01) -> np.ndarray:
    """DOS Chebyshev moments (1/R) sum_r <r|T_n(Ht)|r> / D with random-phase probes."""
    _sync_torch()
    mu = np.zeros(n_moments)
    _check(lib().mb_kpm_dos_moments(op.handle, n_moments, n_probes, seed, e_min, e_max, padding,
                                    mu.ctypes.data_as(_dp)))
    return mu


def jackson_kernel(n: int) -> np.ndarray:
    g = np.zeros(n + 1)
    _check(lib().mb_kpm_jackson_kernel(n, g.ctypes.data_as(_dp)))
    return g


def lorentz_kernel(n: int, lam: float = 4.0) -> np.ndarray:
    g = np.zeros(n + 1)
    _check(lib().mb_kpm_lorentz_kernel(n, lam, g.ctypes.data_as(_dp)))
    return g


class SparseKPMProjector:
    """kpm::SparseKPMProjector (src/numerics/kpm.h:184-241) over the GPU operator."""

    def __init__(self, op: GpuHubbardOperator, expansion_order: int, e_min: float, e_max: float,
                 e_fermi: float = 0.0, padding: float = 0.01):
        self.op, self.M = op, expansion_order
        self.e_min, self.e_max, self.e_fermi, self.padding = e_min, e_max, e_fermi, padding

    def dimension(self) -> int:
        return self.op.dimension()

    def apply(self, v, order: int = ORDER_REFERENCE, out=None):
        _sync_torch()
        y = self.op.empty() if out is None else out
        _check(lib().mb_kpm_projector_apply(self.op.handle, self.M, self.e_min, self.e_max,
                                            self.e_fermi, self.padding, self.op._v(v), order, self.op._v(y)))
        return y


def estimate_bounds(op: GpuHubbardOperator, power_iterations: int, spectral_padding: float,
                    seed: int = 0):
    """estimate_bounds (src/numerics/linear_operator_utils.h:53-77)."""
    _sync_torch()
    lo, hi = C.c_double(), C.c_double()
    _check(lib().mb_estimate_bounds(op.handle, power_iterations, spectral_padding, seed,
                                    C.byref(lo), C.byref(hi)))
    return lo.value, hi.value


# ---------------------------------------------------------------------------
# Batched / served ground states (mb_engine_*).
# ---------------------------------------------------------------------------
def sector(dims, n_up, n_down, t=1.0, u=0.0) -> SectorDesc:
    d = SectorDesc()
    dims = list(dims)
    for i, v in enumerate(dims):
        d.dims[i] = int(v)
    d.ndim = len(dims)
    d.n_up, d.n_down, d.t, d.u = int(n_up), int(n_down), float(t), float(u)
    return d


@dataclass
class EngineResult:
    e0: float
    e0_raw: float
    steps: int
    latency_s: float


class Engine:
    """Many independent sectors advanced together (continuous batching)."""

    def __init__(self, device_bytes_budget: int = 0):
        h = C.c_void_p()
        _check(lib().mb_engine_create(device_bytes_budget, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mb_engine_destroy(self._h)
            self._h = None

    @staticmethod
    def footprint(desc: SectorDesc) -> int:
        b = C.c_int64()
        _check(lib().mb_engine_footprint(C.byref(desc), C.byref(b)))
        return b.value

    def try_submit(self, desc: SectorDesc, seed: int = 0, kmax: int = 200, rel_tol: float = 0.0,
                   refine: bool = True):
        """Request id, or None when the device-memory budget is full."""
        rid = C.c_int64()
        rc = lib().mb_engine_submit_ground_state(self._h, C.byref(desc), seed, kmax, rel_tol,
                                                 int(refine), C.byref(rid))
        if rc == MB_ERR_CAPACITY:
            return None
        _check(rc)
        return rid.value

    def try_submit_dos(self, desc: SectorDesc, n_moments: int = 512, n_probes: int = 1,
                       seed: int = 0, padding: float = 0.01):
        """DOS-moment request id, or None when the device-memory budget is full."""
        rid = C.c_int64()
        rc = lib().mb_engine_submit_dos(self._h, C.byref(desc), n_moments, n_probes, seed, padding,
                                        C.byref(rid))
        if rc == MB_ERR_CAPACITY:
            return None
        _check(rc)
        self._dos_moments = getattr(self, "_dos_moments", {})
        self._dos_moments[rid.value] = n_moments
        return rid.value

    def poll_dos(self, rid: int):
        """(mu, e_min, e_max, latency_s) once finished, else None."""
        n = self._dos_moments[rid]
        mu = np.zeros(n)
        done = C.c_int()
        lo, hi, lat = C.c_double(), C.c_double(), C.c_double()
        _check(lib().mb_engine_poll_dos(self._h, rid, C.byref(done), mu.ctypes.data_as(_dp),
                                        C.byref(lo), C.byref(hi), C.byref(lat)))
        return (mu, lo.value, hi.value, lat.value) if done.value else None

    def step(self, n: int = 1) -> int:
        a = C.c_int()
        _check(lib().mb_engine_step(self._h, n, C.byref(a)))
        return a.value

    def step_fixed(self, n: int, use_graph: bool = True) -> int:
        a = C.c_int()
        _check(lib().mb_engine_step_fixed(self._h, n, int(use_graph), C.byref(a)))
        return a.value

    def poll(self, rid: int):
        done = C.c_int()
        e0, er, lat = C.c_double(), C.c_double(), C.c_double()
        st = C.c_int64()
        _check(lib().mb_engine_poll(self._h, rid, C.byref(done), C.byref(e0), C.byref(er),
                                    C.byref(st), C.byref(lat)))
        return EngineResult(e0.value, er.value, st.value, lat.value) if done.value else None

    def set_warps(self, w: int):
        _check(lib().mb_engine_set_warps(self._h, w))

    def completed(self, capacity: int = 4096):
        """Ids of requests finished since the last call (oldest first)."""
        ids = np.zeros(capacity, np.int64)
        n = C.c_int64()
        _check(lib().mb_engine_completed(self._h, ids.ctypes.data_as(_i64p), capacity, C.byref(n)))
        return [int(i) for i in ids[:n.value]]

    def stats(self):
        """(steps, wall ms, device ms) summed over step() calls."""
        st = C.c_int64()
        w, d = C.c_double(), C.c_double()
        _check(lib().mb_engine_stats(self._h, C.byref(st), C.byref(w), C.byref(d)))
        return st.value, w.value, d.value

    def set_persistent(self, on: bool):
        """The persistent fused step (default) or the grouped kernels."""
        _check(lib().mb_engine_set_persistent(self._h, int(bool(on))))

    def set_basis_limit(self, nbytes: int):
        """Largest pass-one Lanczos basis a ground-state request keeps (0: replay)."""
        _check(lib().mb_engine_set_basis_limit(self._h, int(nbytes)))

    def set_wait_budget(self, cycles: int):
        """clock64 budget of one grid-barrier wait of the persistent step."""
        _check(lib().mb_engine_set_wait_budget(self._h, int(cycles)))

    def shape(self) -> dict:
        sh = EngineShape()
        _check(lib().mb_engine_get_shape(self._h, C.byref(sh)))
        return {"persistent": sh.persistent, "row_min_cols": sh.row_min_cols,
                "ctas_per_sm": sh.ctas_per_sm, "grid": sh.grid, "warps": sh.warps}

    def set_shape(self, persistent=None, row_min_cols=None, ctas_per_sm=None, warps=None):
        cur = self.shape()
        sh = EngineShape()
        sh.persistent = cur["persistent"] if persistent is None else int(bool(persistent))
        sh.row_min_cols = cur["row_min_cols"] if row_min_cols is None else row_min_cols
        sh.ctas_per_sm = cur["ctas_per_sm"] if ctas_per_sm is None else ctas_per_sm
        sh.warps = cur["warps"] if warps is None else warps
        _check(lib().mb_engine_set_shape(self._h, C.byref(sh)))

    def set_fused_threshold(self, min_states: int):
        """Sectors of at least min_states states use the fused complex64 apply."""
        _check(lib().mb_engine_set_fused_threshold(self._h, min_states))

    def autotune(self):
        w, ms = C.c_int(), C.c_double()
        _check(lib().mb_engine_autotune(self._h, C.byref(w), C.byref(ms)))
        return w.value, ms.value


def batch_ground_states(descs, seeds=None, kmax: int = 150, refine: bool = True,
                        use_graph: bool = True, autotune: bool = True, fused_threshold=None,
                        persistent: bool = True, engine_out=None, basis_limit=None,
                        engine=None):
    """Fixed-length batched Lanczos for many sectors: returns [EngineResult].
    engine: run on this Engine (its memory pool and sector tables stay warm
    from earlier batches) instead of a new one."""
    eng = engine if engine is not None else Engine()
    if engine_out is not None:
        engine_out.append(eng)
    if not persistent:
        eng.set_persistent(False)
    if basis_limit is not None:
        eng.set_basis_limit(basis_limit)
    if fused_threshold is not None:
        eng.set_fused_threshold(fused_threshold)
    seeds = seeds if seeds is not None else [0] * len(descs)
    ids = []
    for d, s in zip(descs, seeds):
        rid = eng.try_submit(d, s, kmax, 0.0, refine)
        if rid is None:
            raise MbError(MB_ERR_CAPACITY, "batch does not fit the device-memory budget")
        ids.append(rid)
    if autotune:
        eng.autotune()
    eng.step_fixed(kmax, use_graph)           # pass one (all requests, kmax steps)
    while eng.step_fixed(kmax, use_graph):    # replay + refinement
        pass
    return [eng.poll(i) for i in ids]
