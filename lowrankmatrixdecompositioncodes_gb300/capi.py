"""ctypes mirror of RSVDPACK's C API.

The reference exposes plain C: column-major ``mat``/``vec`` structs
(multi_core_mkl_code/matrix_vector_functions_intel_mkl.h:18-27) and the
decomposition routines of multi_core_mkl_code/rank_revealing_algorithms_intel_mkl.h.
``RsvdLibrary`` binds any shared library that exports that API -- the GPU engine
(librsvdpack.so), or a CPU build of the same API -- and offers numpy-in /
numpy-out wrappers with the reference's names, argument meanings and output
conventions (0-based indices returned as float64, S as a dense k x k matrix,
singular-value order as the reference gives it).

Ownership follows the reference: inputs are borrowed, outputs are allocated by the
callee with ``matrix_new``/``vector_new`` and released here with
``matrix_delete``/``vector_delete`` after copying into numpy.

``RsvdLibrary(path, index64=True)`` binds the int64_t-dimension form of the same API
(multi_core_mkl_code_64bit/matrix_vector_functions_intel_mkl.h:20-28 and
rank_revealing_algorithms_intel_mkl.h), which librsvdpack64.so exports;
``RsvdLibrary(path, real32=True)`` the float-data, int64_t-dimension form of the oneAPI variant
(oneapi_code/matrix_vector_functions_one_api.h:19-32, float TOL), which librsvdpack_f32.so
exports: numpy inputs are rounded to float32 and outputs come back as float32.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np


class Mat(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("d", C.POINTER(C.c_double))]


class Vec(C.Structure):
    _fields_ = [("nrows", C.c_int), ("d", C.POINTER(C.c_double))]


class Mat64(C.Structure):
    _fields_ = [("nrows", C.c_int64), ("ncols", C.c_int64), ("d", C.POINTER(C.c_double))]


class Vec64(C.Structure):
    _fields_ = [("nrows", C.c_int64), ("d", C.POINTER(C.c_double))]


class MatF32(C.Structure):
    _fields_ = [("nrows", C.c_int64), ("ncols", C.c_int64), ("d", C.POINTER(C.c_float))]


class VecF32(C.Structure):
    _fields_ = [("nrows", C.c_int64), ("d", C.POINTER(C.c_float))]


PMat = C.POINTER(Mat)
PVec = C.POINTER(Vec)
OMEGA_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double))

def _algos(_I, PMat, PVec, _D=C.c_double):
    """name -> argtypes for the reference API (rank_revealing_algorithms_intel_mkl.h:3-110),
    with index type _I (c_int, or c_int64 for the 64-bit forms) and TOL type _D (c_double, or
    c_float for the oneAPI form)."""
    _PI = C.POINTER(_I)
    _PPM = C.POINTER(PMat)
    _PPV = C.POINTER(PVec)
    return {
        "low_rank_svd_rand_decomp_fixed_rank": [PMat, _I, _I, _I, _I, _I, _PI, _PPM, _PPM, _PPM],
        "low_rank_svd_blockrand_decomp_fixed_rank_or_prec":
            [PMat, _I, _I, _D, _I, _I, _I, _I, _PI, _PPM, _PPM, _PPM],
        "randQB_pb_new": [PMat, _I, _I, _D, _I, _I, _PI, _PPM, _PPM],
        "randQB_pb2": [PMat, _I, _I, _D, _I, _I, _PI, _PPM, _PPM],
        "randQB_pb": [PMat, _I, _I, _I, _I, _PPM, _PPM],
        "pivotedQR_mkl": [PMat, _PPM, _PPM, _PPV],
        "pivoted_QR_of_specified_rank_or_prec": [PMat, _I, _D, _PI, _PPM, _PPM, _PPV],
        "pivoted_QR_of_specified_rank": [PMat, _I, _PI, _PPM, _PPM, _PPV],
        "id_decomp_fixed_rank_or_prec": [PMat, _I, _D, _PI, _PPV, _PPM],
        "id_rand_decomp_fixed_rank": [PMat, _I, _I, _I, _I, _PPV, _PPM],
        "id_blockrand_decomp_fixed_rank_or_prec": [PMat, _I, _I, _D, _I, _I, _I, _PI, _PPV, _PPM],
        "id_two_sided_decomp_fixed_rank_or_prec": [PMat, _I, _D, _PI, _PPV, _PPV, _PPM, _PPM],
        "id_two_sided_rand_decomp_fixed_rank": [PMat, _I, _I, _I, _I, _PPV, _PPV, _PPM, _PPM],
        "id_two_sided_blockrand_decomp_fixed_rank_or_prec":
            [PMat, _I, _I, _D, _I, _I, _I, _PI, _PPV, _PPV, _PPM, _PPM],
        "cur_decomp_fixed_rank_or_prec": [PMat, _I, _D, _PI, _PPM, _PPM, _PPM],
        "cur_rand_decomp_fixed_rank": [PMat, _I, _I, _I, _I, _PPM, _PPM, _PPM],
        "cur_blockrand_decomp_fixed_rank_or_prec":
            [PMat, _I, _I, _D, _I, _I, _I, _PI, _PPM, _PPM, _PPM],
        # the QB split of the oneAPI variant (oneapi_code/rank_revealing_algorithms_one_api.h:6,10)
        "low_rank_svd_rand_decomp_fromQB": [PMat, PMat, _PPM, _PPM, _PPM],
        "id_rand_decomp_fromQB": [PMat, PMat, _PPV, _PPM],
    }


class SeededOmega:
    """Gaussian test matrices from a seed: request c of N values is
    ``default_rng([seed, c]).standard_normal(N)`` rounded through float32 (the
    reference draws float Gaussians, matrix_vector_functions_intel_mkl.c:458-486).
    Values depend on the element count only, not on the requested shape."""

    def __init__(self, seed: int = 0):
        self.seed = int(seed)
        self.served: list[np.ndarray] = []
        self.record = False

    def __call__(self, call_index: int, count: int) -> np.ndarray:
        g = np.random.default_rng([self.seed, int(call_index)])
        v = g.standard_normal(count).astype(np.float32)
        if self.record:
            self.served.append(v.copy())
        return v


class ListOmega:
    """Serves a fixed list of float32 arrays, one per request, in order."""

    def __init__(self, arrays):
        self.arrays = [np.asarray(a, dtype=np.float32).ravel() for a in arrays]

    def __call__(self, call_index: int, count: int) -> np.ndarray:
        a = self.arrays[call_index]
        if a.size != count:
            raise ValueError(f"omega request {call_index}: want {count} values, have {a.size}")
        return a


_ALGOS = _algos(C.c_int, PMat, PVec)


class RsvdLibrary:
    """Binds one shared library exporting the reference C API: LP64 int dimensions, or
    int64_t dimensions with ``index64=True``."""

    def __init__(self, path: str, index64: bool = False, real32: bool = False):
        self.path = str(path)
        self.real32 = bool(real32)
        self.index64 = bool(index64) or self.real32
        self.Int = C.c_int64 if self.index64 else C.c_int
        self.Real = C.c_float if self.real32 else C.c_double
        self.dtype = np.float32 if self.real32 else np.float64
        if self.real32:
            self.Mat, self.Vec = MatF32, VecF32
        else:
            self.Mat = Mat64 if self.index64 else Mat
            self.Vec = Vec64 if self.index64 else Vec
        self.PMat = C.POINTER(self.Mat)
        self.PVec = C.POINTER(self.Vec)
        PMat, PVec, _I, _D = self.PMat, self.PVec, self.Int, self.Real
        self.lib = C.CDLL(self.path)
        L = self.lib
        L.matrix_new.restype = PMat
        L.matrix_new.argtypes = [_I, _I]
        L.vector_new.restype = PVec
        L.vector_new.argtypes = [_I]
        L.matrix_delete.argtypes = [PMat]
        L.vector_delete.argtypes = [PVec]
        L.matrix_delete.restype = None
        L.vector_delete.restype = None
        L.get_matrix_frobenius_norm.restype = _D
        L.get_matrix_frobenius_norm.argtypes = [PMat]
        L.get_percent_error_between_two_mats.restype = _D
        L.get_percent_error_between_two_mats.argtypes = [PMat, PMat]
        for name, args in _algos(_I, PMat, PVec, _D).items():
            f = getattr(L, name, None)
            if f is not None:
                f.argtypes = args
                f.restype = None
        L.rsvdpack_set_omega_provider.argtypes = [OMEGA_FN, C.c_void_p]
        L.rsvdpack_set_omega_provider.restype = None
        L.rsvdpack_reset_omega_counter.argtypes = []
        L.rsvdpack_reset_omega_counter.restype = None
        L.rsvdpack_omega_calls.restype = C.c_int
        self._omega_cb = None
        self._omega = None

    # ---------------------------------------------------------------- helpers
    def has(self, name: str) -> bool:
        return hasattr(self.lib, name)

    def to_mat(self, A):
        A = np.asarray(A, dtype=self.dtype)
        if A.ndim != 2:
            raise ValueError("matrix must be 2-D")
        m, n = A.shape
        pM = self.lib.matrix_new(m, n)
        if m * n:
            buf = np.ctypeslib.as_array(pM.contents.d, shape=(m * n,))
            buf[:] = A.ravel(order="F")
        return pM

    def from_mat(self, pM, free: bool = True) -> np.ndarray:
        m, n = pM.contents.nrows, pM.contents.ncols
        if m * n:
            out = np.ctypeslib.as_array(pM.contents.d, shape=(m * n,)).copy()
            out = out.reshape((m, n), order="F")
        else:
            out = np.zeros((m, n))
        if free:
            self.lib.matrix_delete(pM)
        return out

    def from_vec(self, pv, free: bool = True) -> np.ndarray:
        n = pv.contents.nrows
        out = np.ctypeslib.as_array(pv.contents.d, shape=(n,)).copy() if n else np.zeros(0)
        if free:
            self.lib.vector_delete(pv)
        return out

    def set_omega(self, provider: Optional[Callable[[int, int], np.ndarray]]):
        """Register the Gaussian test-matrix provider (None: library default)."""
        if provider is None:
            self._omega_cb = None
            self._omega = None
            self.lib.rsvdpack_set_omega_provider(OMEGA_FN(), None)
            return

        def _cb(ctx, call_index, nrows, ncols, out):
            count = int(nrows) * int(ncols)
            vals = provider(int(call_index), count)
            np.ctypeslib.as_array(out, shape=(count,))[:] = vals

        self._omega = provider
        self._omega_cb = OMEGA_FN(_cb)
        self.lib.rsvdpack_set_omega_provider(self._omega_cb, None)

    def omega_calls(self) -> int:
        return int(self.lib.rsvdpack_omega_calls())

    def _call(self, name, M, *scalars, nm=0, nv=0, frank=False):
        pm = [self.PMat() for _ in range(nm)]
        pv = [self.PVec() for _ in range(nv)]
        fr = self.Int(-1)
        args = [M, *scalars]
        if frank:
            args.append(C.byref(fr))
        return pm, pv, fr, args

    # ------------------------------------------------------------ algorithms
    def low_rank_svd_rand_decomp_fixed_rank(self, A, k, p, vnum, q, s):
        M = self.to_mat(A)
        U, S, V, fr = self.PMat(), self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.low_rank_svd_rand_decomp_fixed_rank(
                M, k, p, vnum, q, s, C.byref(fr), C.byref(U), C.byref(S), C.byref(V))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(U), self.from_mat(S), self.from_mat(V)

    def low_rank_svd_blockrand_decomp_fixed_rank_or_prec(self, A, k, p, TOL, vnum, kstep, q, s):
        M = self.to_mat(A)
        U, S, V, fr = self.PMat(), self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.low_rank_svd_blockrand_decomp_fixed_rank_or_prec(
                M, k, p, float(TOL), vnum, kstep, q, s, C.byref(fr),
                C.byref(U), C.byref(S), C.byref(V))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(U), self.from_mat(S), self.from_mat(V), fr.value

    def randQB_pb_new(self, A, kstep, nstep, TOL, q, s):
        M = self.to_mat(A)
        Q, B, fr = self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.randQB_pb_new(M, kstep, nstep, float(TOL), q, s, C.byref(fr),
                                   C.byref(Q), C.byref(B))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Q), self.from_mat(B), fr.value

    def randQB_pb2(self, A, kstep, nstep, TOL, q, s):
        M = self.to_mat(A)
        Q, B, fr = self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.randQB_pb2(M, kstep, nstep, float(TOL), q, s, C.byref(fr), C.byref(Q), C.byref(B))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Q), self.from_mat(B), fr.value

    def randQB_pb(self, A, kstep, nstep, q, s):
        M = self.to_mat(A)
        Q, B = self.PMat(), self.PMat()
        try:
            self.lib.randQB_pb(M, kstep, nstep, q, s, C.byref(Q), C.byref(B))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Q), self.from_mat(B)

    def low_rank_svd_rand_decomp_fromQB(self, Qm, Bm):
        Q, B = self.to_mat(Qm), self.to_mat(Bm)
        U, S, V = self.PMat(), self.PMat(), self.PMat()
        try:
            self.lib.low_rank_svd_rand_decomp_fromQB(Q, B, C.byref(U), C.byref(S), C.byref(V))
        finally:
            self.lib.matrix_delete(Q)
            self.lib.matrix_delete(B)
        return self.from_mat(U), self.from_mat(S), self.from_mat(V)

    def id_rand_decomp_fromQB(self, Qm, Bm):
        Q, B = self.to_mat(Qm), self.to_mat(Bm)
        I, T = self.PVec(), self.PMat()
        try:
            self.lib.id_rand_decomp_fromQB(Q, B, C.byref(I), C.byref(T))
        finally:
            self.lib.matrix_delete(Q)
            self.lib.matrix_delete(B)
        return self.from_vec(I), self.from_mat(T)

    def pivotedQR_mkl(self, A):
        M = self.to_mat(A)
        Q, R, I = self.PMat(), self.PMat(), self.PVec()
        try:
            self.lib.pivotedQR_mkl(M, C.byref(Q), C.byref(R), C.byref(I))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Q), self.from_mat(R), self.from_vec(I)

    def pivoted_QR_of_specified_rank_or_prec(self, A, k, TOL):
        M = self.to_mat(A)
        Q, R, I, fr = self.PMat(), self.PMat(), self.PVec(), self.Int(-1)
        try:
            self.lib.pivoted_QR_of_specified_rank_or_prec(
                M, k, float(TOL), C.byref(fr), C.byref(Q), C.byref(R), C.byref(I))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Q), self.from_mat(R), self.from_vec(I), fr.value

    def pivoted_QR_of_specified_rank(self, A, k):
        M = self.to_mat(A)
        Q, R, I, fr = self.PMat(), self.PMat(), self.PVec(), self.Int(-1)
        try:
            self.lib.pivoted_QR_of_specified_rank(M, k, C.byref(fr), C.byref(Q), C.byref(R), C.byref(I))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Q), self.from_mat(R), self.from_vec(I), fr.value

    def id_decomp_fixed_rank_or_prec(self, A, k, TOL):
        M = self.to_mat(A)
        I, T, fr = self.PVec(), self.PMat(), self.Int(-1)
        try:
            self.lib.id_decomp_fixed_rank_or_prec(M, k, float(TOL), C.byref(fr),
                                                  C.byref(I), C.byref(T))
        finally:
            self.lib.matrix_delete(M)
        return self.from_vec(I), self.from_mat(T), fr.value

    def id_rand_decomp_fixed_rank(self, A, k, p, q, s):
        M = self.to_mat(A)
        I, T = self.PVec(), self.PMat()
        try:
            self.lib.id_rand_decomp_fixed_rank(M, k, p, q, s, C.byref(I), C.byref(T))
        finally:
            self.lib.matrix_delete(M)
        return self.from_vec(I), self.from_mat(T)

    def id_blockrand_decomp_fixed_rank_or_prec(self, A, k, p, TOL, kstep, q, s):
        M = self.to_mat(A)
        I, T, fr = self.PVec(), self.PMat(), self.Int(-1)
        try:
            self.lib.id_blockrand_decomp_fixed_rank_or_prec(
                M, k, p, float(TOL), kstep, q, s, C.byref(fr), C.byref(I), C.byref(T))
        finally:
            self.lib.matrix_delete(M)
        return self.from_vec(I), self.from_mat(T), fr.value

    def id_two_sided_decomp_fixed_rank_or_prec(self, A, k, TOL):
        M = self.to_mat(A)
        Ic, Ir, T, S, fr = self.PVec(), self.PVec(), self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.id_two_sided_decomp_fixed_rank_or_prec(
                M, k, float(TOL), C.byref(fr), C.byref(Ic), C.byref(Ir), C.byref(T), C.byref(S))
        finally:
            self.lib.matrix_delete(M)
        return (self.from_vec(Ic), self.from_vec(Ir), self.from_mat(T), self.from_mat(S),
                fr.value)

    def id_two_sided_rand_decomp_fixed_rank(self, A, k, p, q, s):
        M = self.to_mat(A)
        Ic, Ir, T, S = self.PVec(), self.PVec(), self.PMat(), self.PMat()
        try:
            self.lib.id_two_sided_rand_decomp_fixed_rank(
                M, k, p, q, s, C.byref(Ic), C.byref(Ir), C.byref(T), C.byref(S))
        finally:
            self.lib.matrix_delete(M)
        return self.from_vec(Ic), self.from_vec(Ir), self.from_mat(T), self.from_mat(S)

    def id_two_sided_blockrand_decomp_fixed_rank_or_prec(self, A, k, p, TOL, kstep, q, s):
        M = self.to_mat(A)
        Ic, Ir, T, S, fr = self.PVec(), self.PVec(), self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.id_two_sided_blockrand_decomp_fixed_rank_or_prec(
                M, k, p, float(TOL), kstep, q, s, C.byref(fr), C.byref(Ic), C.byref(Ir),
                C.byref(T), C.byref(S))
        finally:
            self.lib.matrix_delete(M)
        return (self.from_vec(Ic), self.from_vec(Ir), self.from_mat(T), self.from_mat(S),
                fr.value)

    def cur_decomp_fixed_rank_or_prec(self, A, k, TOL):
        M = self.to_mat(A)
        Cm, U, R, fr = self.PMat(), self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.cur_decomp_fixed_rank_or_prec(M, k, float(TOL), C.byref(fr),
                                                   C.byref(Cm), C.byref(U), C.byref(R))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Cm), self.from_mat(U), self.from_mat(R), fr.value

    def cur_rand_decomp_fixed_rank(self, A, k, p, q, s):
        M = self.to_mat(A)
        Cm, U, R = self.PMat(), self.PMat(), self.PMat()
        try:
            self.lib.cur_rand_decomp_fixed_rank(M, k, p, q, s, C.byref(Cm), C.byref(U),
                                                C.byref(R))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Cm), self.from_mat(U), self.from_mat(R)

    def cur_blockrand_decomp_fixed_rank_or_prec(self, A, k, p, TOL, kstep, q, s):
        M = self.to_mat(A)
        Cm, U, R, fr = self.PMat(), self.PMat(), self.PMat(), self.Int(-1)
        try:
            self.lib.cur_blockrand_decomp_fixed_rank_or_prec(
                M, k, p, float(TOL), kstep, q, s, C.byref(fr), C.byref(Cm), C.byref(U),
                C.byref(R))
        finally:
            self.lib.matrix_delete(M)
        return self.from_mat(Cm), self.from_mat(U), self.from_mat(R), fr.value
