"""elastic_gb300: GB300-native (sm_103a) linear-elasticity solve path.

Python face of ``libelastic_gb300.so`` (C ABI in ``include/elastic_gb300.h``).
The host-side calls mirror the two routines of lmn-labest/Elastic that the
library replaces -- ``pform_mec`` (mef/src/Pform.f:1-11) and ``solv``
(mef/src/Solv.f:13-15) -- with the same argument meaning (1-based index
contents, Fortran column-major arrays) and the same error behaviour turned
into exceptions: where the reference calls ``stop`` (zero diagonal, no
convergence, non-positive Jacobian) the library returns a status and
:class:`ElasticError` is raised with it.

There is no CPU fallback: if the shared library or a CUDA device is missing,
every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

__all__ = ["ElasticError", "Context", "Server", "Info", "load", "library_path", "pform_mec",
           "solv", "pload", "edge_loads", "host_structure", "host_colors", "host_partition", "fp64_fma_rate",
           "fortran_e",
           "solvm", "SOLVER_PCG", "SOLVER_GMRES", "SOLVER_BICGSTAB", "SOLVER_BICGSTAB_NOPREC", "PREC_FP64",
           "PREC_MIXED", "VTK_VTU_ASCII", "VTK_LEGACY_BINARY", "VTK_DESLOC", "VTK_STRESS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libelastic_gb300.so")

OK, ERR_ZERO_DIAG, ERR_NO_CONVERGENCE, ERR_BAD_DET, ERR_OOM, ERR_TIMEOUT, ERR_ARG, \
    ERR_BAD_ELEMENT, ERR_CUDA, ERR_STATE = range(10)
SOLVER_PCG, SOLVER_GMRES, SOLVER_BICGSTAB, SOLVER_BICGSTAB_NOPREC = 1, 2, 4, 5
PREC_FP64, PREC_MIXED = 0, 1
VTK_VTU_ASCII, VTK_LEGACY_BINARY = 0, 1   # result file formats
VTK_DESLOC, VTK_STRESS = 1, 2             # result fields (fprint(2), fprint(3))

STATUS_NAMES = {0: "ok", 1: "zero diagonal", 2: "no convergence", 3: "bad determinant",
                4: "out of memory", 5: "timeout", 6: "bad argument",
                7: "bad element type", 8: "cuda error", 9: "bad call order"}


class ElasticError(RuntimeError):
    """A non-zero status of the C ABI (the reference would have stopped)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{STATUS_NAMES.get(code, code)}] {msg}")
        self.code = code


class Opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("verbose", C.c_int32), ("hbm_budget", C.c_int64)]


class Info(C.Structure):
    """Post-solve diagnostics (the fields pcg prints, Iters.f:473-490)."""
    _fields_ = [("iters", C.c_int32), ("status", C.c_int32), ("xkx", C.c_double),
                ("norm_x", C.c_double), ("norm_r", C.c_double), ("norm_m_r", C.c_double),
                ("conv", C.c_double), ("seconds", C.c_double), ("mflops", C.c_double),
                ("refinements", C.c_int32), ("inner_iters", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("prep_threads", C.c_int32), ("hbm_budget", C.c_int64),
                ("poll_steps", C.c_int32), ("max_slots", C.c_int32), ("large_dofs", C.c_int32),
                ("large_mode", C.c_int32), ("large_workers", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("peak_bytes", C.c_int64),
                ("resident_bytes", C.c_int64), ("peak_slots", C.c_int64),
                ("iterations", C.c_int64), ("large_solved", C.c_int64),
                ("phase_n", C.c_int64 * 2), ("phase_s", (C.c_double * 5) * 2)]
    PHASES = ("prepare", "wait_admission", "admit", "wait_start", "solve")

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_[:7]}
        # mean seconds per phase of the finished packed / block requests
        for k, kind in enumerate(("packed", "block")):
            n = self.phase_n[k]
            d[f"{kind}_phases_mean_s"] = {
                p: (self.phase_s[k][i] / n if n else None) for i, p in enumerate(self.PHASES)}
            d[f"{kind}_finished"] = n
        return d


_lib = None
_VP = C.c_void_p
_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_F64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def library_path() -> str:
    return _LIB_PATH


def load():
    """Load the shared library (built by ``python -m elastic_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise ElasticError(ERR_STATE, f"{_LIB_PATH} not built; run python -m elastic_gb300.build")
    L = C.CDLL(_LIB_PATH)
    P = C.POINTER
    sig = {
        "elx_version": (C.c_char_p, []),
        "elx_create": (C.c_int, [P(_VP), P(Opts)]),
        "elx_destroy": (None, [_VP]),
        "elx_last_error": (C.c_char_p, [_VP]),
        "elx_stream": (_VP, [_VP]),
        "elx_device_bytes": (C.c_int64, [_VP]),
        "elx_kernel_launches": (C.c_int64, [_VP]),
        "elx_set_mesh": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                   _I32, _F64, _I32, _F64, C.c_int32, C.c_int32]),
        "elx_set_structure": (C.c_int, [_VP, C.c_int32, C.c_int64, _I32, _I32, _VP]),
        "elx_build_structure": (C.c_int, [_VP, _I32, C.c_int32]),
        "elx_get_sizes": (C.c_int, [_VP, P(C.c_int32), P(C.c_int64), P(C.c_int32)]),
        "elx_get_structure": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
        "elx_assemble": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
        "elx_solve": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                _F64, _F64, P(Info)]),
        "elx_update": (C.c_int, [_VP, _F64, _F64]),
        "elx_spmv": (C.c_int, [_VP, C.c_int32, _F64, _F64]),
        "elx_set_matrix": (C.c_int, [_VP, _F64, _VP]),
        "elx_set_state": (C.c_int, [_VP, _VP, _VP]),
        "elx_assemble_resident": (C.c_int, [_VP]),
        "elx_solve_resident": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                         C.c_int32, P(Info)]),
        "elx_spmv_resident": (C.c_int, [_VP, C.c_int32, C.c_int32]),
        "elx_get_solution": (C.c_int, [_VP, _F64]),
        "elx_host_structure_create": (C.c_int, [P(_VP), C.c_int32, C.c_int32, C.c_int32,
                                                C.c_int32, C.c_int32, _I32, _I32, C.c_int32,
                                                _I32, C.c_int32]),
        "elx_host_structure_sizes": (C.c_int, [_VP, P(C.c_int32), P(C.c_int64)]),
        "elx_host_structure_get": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
        "elx_host_structure_colors": (C.c_int, [_VP, _VP, _VP]),
        "elx_host_structure_destroy": (None, [_VP]),
        "elx_get_rhs": (C.c_int, [_VP, _F64]),
        "elx_spmv_dot_noalloc": (C.c_int, [C.c_int32, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                           _VP, _VP, _VP]),
        "elx_solve_block": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                      C.c_int32, _VP, _VP, _VP]),
        "elx_solve_block_device": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                             C.c_int32, _VP, _VP, _VP]),
        "elx_autotune_block": (C.c_int, [_VP, C.c_int32, P(C.c_int32), _VP]),
        "elx_block_tiling": (C.c_int, [_VP, C.c_int32, _VP]),
        "elx_stress": (C.c_int, [_VP, _VP, _VP, _VP]),
        "elx_update_resident": (C.c_int, [_VP]),
        "elx_set_loads": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int32]),
        "elx_partition_spmv": (C.c_int, [_VP, C.c_int32, _VP, _VP]),
        "elx_partition_spmv_resident": (C.c_int, [_VP, C.c_int32, C.c_int32]),
        "elx_partition_info": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP, _VP, _VP]),
        "elx_host_partition_sizes": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP, _VP, _VP, _VP,
                                               _VP]),
        "elx_host_partition_get": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP, _VP, _VP, _VP,
                                             _VP, _VP, _VP]),
        "elx_write_vtk": (C.c_int, [_VP, C.c_char_p, C.c_int32, C.c_int32, _VP]),
        "elx_format_vtk": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP, C.c_int64, _VP]),
        "elx_fortran_e": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _VP]),
        "elx_fp64_fma_rate": (C.c_int, [C.c_int32, _VP, _VP]),
        "elx_get_state": (C.c_int, [_VP, _VP, _VP]),
        "elx_server_create": (C.c_int, [P(_VP), P(ServerOpts)]),
        "elx_server_destroy": (None, [_VP]),
        "elx_server_submit": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_int32, _I32, _F64, _I32, _F64, C.c_int32,
                                        C.c_int32, _I32, C.c_int32, _F64, C.c_double,
                                        C.c_int32, P(C.c_int64)]),
        "elx_server_wait": (C.c_int, [_VP, C.c_int64, C.c_double, _VP, _VP, P(C.c_double)]),
        "elx_server_get_stats": (C.c_int, [_VP, P(ServerStats)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_VP)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class StructureArrays:
    perm: np.ndarray
    id: np.ndarray
    ia: np.ndarray
    ja: np.ndarray
    neq: int
    nad: int
    ncolors: int


def host_structure(mesh, reorder: bool = True) -> StructureArrays:
    """Node graph, RCM, numeq and the lower CSRC pattern computed by the
    library on the host (no GPU needed): elx_host_structure_create."""
    L = load()
    h = _VP()
    st = L.elx_host_structure_create(C.byref(h), mesh.ndm, mesh.ndf, mesh.nen, mesh.numel,
                                     mesh.nnode, _i32(mesh.ix), _i32(mesh.ie), mesh.numat,
                                     _i32(mesh.id), int(reorder))
    if st != OK:
        raise ElasticError(st, "host structure build failed")
    try:
        neq, nad = C.c_int32(), C.c_int64()
        L.elx_host_structure_sizes(h, C.byref(neq), C.byref(nad))
        neq, nad = int(neq.value), int(nad.value)
        perm = np.zeros(mesh.nnode, np.int32)
        idm = np.zeros((mesh.nnode, mesh.ndf), np.int32)
        ia = np.zeros(neq + 1, np.int32)
        ja = np.zeros(max(nad, 1), np.int32)
        L.elx_host_structure_get(h, _ptr(perm), _ptr(idm), _ptr(ia), _ptr(ja))
    finally:
        L.elx_host_structure_destroy(h)
    return StructureArrays(perm, idm, ia, ja[:nad], neq, nad, 0)


def fp64_fma_rate(device: int = 0):
    """(FP64 FMAs per second, per clock per SM at the maximum SM clock) of
    the device, from the library's register-only probe kernel."""
    L = load()
    rate, per = C.c_double(), C.c_double()
    st = L.elx_fp64_fma_rate(device, C.byref(rate), C.byref(per))
    if st != OK:
        raise ElasticError(st, "FP64 rate probe failed")
    return rate.value, per.value


def host_colors(mesh) -> np.ndarray:
    """The element colours of the library's assembly (1-based, one per
    element in element order): elx_host_structure_colors."""
    L = load()
    h = _VP()
    st = L.elx_host_structure_create(C.byref(h), mesh.ndm, mesh.ndf, mesh.nen, mesh.numel,
                                     mesh.nnode, _i32(mesh.ix), _i32(mesh.ie), mesh.numat,
                                     _i32(mesh.id), 1)
    if st != OK:
        raise ElasticError(st, "host structure build failed")
    try:
        col = np.zeros(mesh.numel, np.int32)
        nc = C.c_int32()
        st = L.elx_host_structure_colors(h, _ptr(col), C.byref(nc))
        if st != OK:
            raise ElasticError(st, "element colouring failed")
    finally:
        L.elx_host_structure_destroy(h)
    assert col.max() == nc.value
    return col


@dataclass
class PartitionArrays:
    eq0: int
    neq: int
    halo: np.ndarray
    ia: np.ndarray
    ja: np.ndarray
    ia1: np.ndarray
    ja1: np.ndarray
    pos: np.ndarray
    pos1: np.ndarray


def host_partition(mesh, nparts: int, part: int, reorder: bool = True) -> PartitionArrays:
    """Partition `part` of `nparts` row blocks of the library's host structure
    (elx_host_partition_*): the reference's overlapping-partition CSRC with
    its rectangular part, local numbering, halo and value positions."""
    L = load()
    h = _VP()
    st = L.elx_host_structure_create(C.byref(h), mesh.ndm, mesh.ndf, mesh.nen, mesh.numel,
                                     mesh.nnode, _i32(mesh.ix), _i32(mesh.ie), mesh.numat,
                                     _i32(mesh.id), int(reorder))
    if st != OK:
        raise ElasticError(st, "host structure build failed")
    try:
        eq0, neq, nh = C.c_int32(), C.c_int32(), C.c_int32()
        nad, nad1 = C.c_int64(), C.c_int64()
        st = L.elx_host_partition_sizes(h, nparts, part, C.byref(eq0), C.byref(neq),
                                        C.byref(nh), C.byref(nad), C.byref(nad1))
        if st != OK:
            raise ElasticError(st, "host partition failed")
        n = neq.value
        halo = np.zeros(max(nh.value, 1), np.int32)
        ia, ia1 = np.zeros(n + 1, np.int32), np.zeros(n + 1, np.int32)
        ja = np.zeros(max(nad.value, 1), np.int32)
        ja1 = np.zeros(max(nad1.value, 1), np.int32)
        pos = np.zeros(max(nad.value, 1), np.int64)
        pos1 = np.zeros(max(nad1.value, 1), np.int64)
        L.elx_host_partition_get(h, nparts, part, _ptr(halo), _ptr(ia), _ptr(ja), _ptr(ia1),
                                 _ptr(ja1), _ptr(pos), _ptr(pos1))
    finally:
        L.elx_host_structure_destroy(h)
    return PartitionArrays(eq0.value, n, halo[:nh.value], ia, ja[:nad.value], ia1,
                           ja1[:nad1.value], pos[:nad.value], pos1[:nad1.value])


class Context:
    """One device context: mesh, CSRC structure, matrix and solver state
    resident on one GPU."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, verbose: int = 0):
        L = load()
        self._L = L
        h = _VP()
        opts = Opts(device, verbose, hbm_budget)
        st = L.elx_create(C.byref(h), C.byref(opts))
        self._h = h
        if st != OK:
            msg = L.elx_last_error(h).decode() if h else "context creation failed"
            self.close()
            raise ElasticError(st, msg)
        self.mesh = None

    # -- plumbing
    def _check(self, st):
        if st != OK:
            raise ElasticError(st, self._L.elx_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.elx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self._L.elx_stream(self._h) or 0)

    @property
    def device_bytes(self) -> int:
        return int(self._L.elx_device_bytes(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(self._L.elx_kernel_launches(self._h))

    # -- mesh and structure
    def set_mesh(self, mesh):
        self.mesh = mesh
        self._ix = _i32(mesh.ix)
        self._x = _f64(mesh.x)
        self._ie = _i32(mesh.ie)
        self._e = _f64(mesh.e)
        self._check(self._L.elx_set_mesh(self._h, mesh.ndm, mesh.ndf, mesh.nen, mesh.numel,
                                         mesh.nnode, self._ix, self._x, self._ie, self._e,
                                         self._e.shape[1], self._e.shape[0]))

    def build_structure(self, reorder: bool = True):
        """Graph, RCM, numeq and the CSRC pattern computed by the library."""
        self._check(self._L.elx_build_structure(self._h, _i32(self.mesh.id), int(reorder)))
        return self.sizes()

    def set_structure(self, id, ia, ja):
        """Structure computed by the caller (the reference driver's arrays)."""
        id = _i32(id)
        ia = _i32(ia)
        ja = _i32(ja)
        neq = ia.shape[0] - 1
        nad = int(ia[-1]) - 1
        self._check(self._L.elx_set_structure(self._h, neq, nad, id, ia, _ptr(ja)))
        return self.sizes()

    def sizes(self):
        neq, nad, nc = C.c_int32(), C.c_int64(), C.c_int32()
        self._check(self._L.elx_get_sizes(self._h, C.byref(neq), C.byref(nad), C.byref(nc)))
        return int(neq.value), int(nad.value), int(nc.value)

    def structure(self) -> StructureArrays:
        neq, nad, nc = self.sizes()
        m = self.mesh
        perm = np.zeros(m.nnode, np.int32)
        idm = np.zeros((m.nnode, m.ndf), np.int32)
        ia = np.zeros(neq + 1, np.int32)
        ja = np.zeros(max(nad, 1), np.int32)
        self._check(self._L.elx_get_structure(self._h, _ptr(perm), _ptr(idm), _ptr(ia),
                                              _ptr(ja)))
        return StructureArrays(perm, idm, ia, ja[:nad], neq, nad, nc)

    # -- assembly and solve
    def assemble(self, u=None, b0=None, want_matrix=False):
        """pform_mec(isw=2): returns b = b0 - K u, and (ad, al) if asked."""
        neq, nad, _ = self.sizes()
        u = None if u is None else _f64(u)
        b0 = None if b0 is None else _f64(b0)
        b = np.zeros(neq)
        ad = np.zeros(neq) if want_matrix else None
        al = np.zeros(max(nad, 1)) if want_matrix else None
        self._check(self._L.elx_assemble(self._h, _ptr(u), _ptr(b0), _ptr(b), _ptr(ad),
                                         _ptr(al)))
        if want_matrix:
            return b, ad, al[:nad]
        return b

    def set_matrix(self, ad, al):
        self._ad_keep, self._al_keep = _f64(ad), _f64(al)
        self._check(self._L.elx_set_matrix(self._h, self._ad_keep, _ptr(self._al_keep)))

    def solve(self, b, solver=SOLVER_PCG, precision=PREC_FP64, tol=1e-11, maxit=10000,
              ngram=50, raise_on_error=True):
        """solv: x with K x = b; returns (x, info dict)."""
        neq, _, _ = self.sizes()
        x = np.zeros(neq)
        info = Info()
        st = self._L.elx_solve(self._h, solver, precision, tol, maxit, ngram, _f64(b), x,
                               C.byref(info))
        if raise_on_error:
            self._check(st)
        d = info.as_dict()
        d["status"] = st if st != OK else d["status"]
        return x, d

    def stress(self, u=None, tx0=None):
        """tform_mec: nodal stresses (nnode, ntn) from nodal displacements u
        (nnode, ndf; None: the resident u) and initial stresses tx0."""
        m = self.mesh
        ntn = 4 if m.ndm == 2 else 6
        t = np.zeros((m.nnode, ntn))
        uu = None if u is None else _f64(u)
        tt = None if tx0 is None else _f64(tx0)
        self._check(self._L.elx_stress(self._h, _ptr(uu), _ptr(tt), t.ctypes.data_as(_VP)))
        return t

    def solve_block(self, B, precision=PREC_MIXED, tol=1e-8, maxit=20000, width=0,
                    raise_on_error=True):
        """Block PCG for the columns of B (neq x nrhs): returns (X, infos)."""
        B = np.asfortranarray(B, dtype=np.float64)
        if B.ndim == 1:
            B = B[:, None]
        neq, nrhs = B.shape
        X = np.zeros((neq, nrhs), order="F")
        infos = (Info * nrhs)()
        st = self._L.elx_solve_block(self._h, nrhs, precision, tol, maxit, width,
                                     B.ctypes.data_as(_VP), X.ctypes.data_as(_VP), infos)
        if raise_on_error:
            self._check(st)
        return X, [i.as_dict() for i in infos]

    def solve_block_device(self, b_ptr, x_ptr, nrhs, precision=PREC_MIXED, tol=1e-8,
                           maxit=20000, width=0):
        """Block PCG on device arrays (pointers to neq x nrhs column-major)."""
        infos = (Info * nrhs)()
        self._check(self._L.elx_solve_block_device(self._h, nrhs, precision, tol, maxit, width,
                                                   _VP(b_ptr), _VP(x_ptr), infos))
        return [i.as_dict() for i in infos]

    def autotune_block(self, precision=PREC_MIXED, remeasure=False):
        """(width, product times in us for widths 1, 2, 4, 8, 16 or None)."""
        w = C.c_int32(0)
        t = np.zeros(5)
        self._check(self._L.elx_autotune_block(self._h, precision, C.byref(w),
                                               t.ctypes.data_as(_VP) if remeasure else None))
        return w.value, (t if remeasure else None)

    def block_tiling(self, precision=PREC_MIXED):
        """The autotuner's slot groups in flight of the block product for
        widths 1, 2, 4, 8, 16 (0: not tuned)."""
        u = np.zeros(5, np.int32)
        self._check(self._L.elx_block_tiling(self._h, precision, u.ctypes.data_as(_VP)))
        return u.tolist()

    def spmv(self, x, precision=PREC_FP64):
        neq, _, _ = self.sizes()
        y = np.zeros(neq)
        self._check(self._L.elx_spmv(self._h, precision, _f64(x), y))
        return y

    def update(self, x, u):
        """update_mec: u(j,i) = x(id(j,i)) for free dofs (a new array)."""
        u = _f64(u).copy()
        self._check(self._L.elx_update(self._h, _f64(x), u))
        return u

    # -- resident (no host copies) steps
    def set_state(self, u=None, b0=None):
        self._check(self._L.elx_set_state(self._h, _ptr(None if u is None else _f64(u)),
                                          _ptr(None if b0 is None else _f64(b0))))

    def set_loads(self, f, eload=None, loadvec=None):
        """pload_mec + the 2-D edge loads (isw = 4) on the device, into the
        resident b0 and u: f (nnode, ndf) evaluated nodal loads, eload
        (numel, 7) 1-based load numbers per side, loadvec (nload, 2)."""
        ff = _f64(f)
        el = None if eload is None else np.ascontiguousarray(eload, dtype=np.int32)
        lv = None if loadvec is None else _f64(np.asarray(loadvec, np.float64).reshape(-1, 2))
        nload = 0 if lv is None else lv.shape[0]
        self._check(self._L.elx_set_loads(self._h, _ptr(ff), _ptr(el), _ptr(lv), nload))

    def format_vtk(self, fmt=VTK_VTU_ASCII, fields=VTK_DESLOC | VTK_STRESS) -> bytes:
        """write_mesh_res_mec's file, formatted on the GPU, as bytes."""
        n = C.c_int64(0)
        self._check(self._L.elx_format_vtk(self._h, fmt, fields, None, 0, C.byref(n)))
        buf = C.create_string_buffer(max(n.value, 1))
        self._check(self._L.elx_format_vtk(self._h, fmt, fields, C.cast(buf, _VP), n.value,
                                           C.byref(n)))
        return buf.raw[:n.value]

    def write_vtk(self, path, fmt=VTK_VTU_ASCII, fields=VTK_DESLOC | VTK_STRESS) -> int:
        """write_mesh_res_mec: the result file at `path`; returns its size."""
        n = C.c_int64(0)
        self._check(self._L.elx_write_vtk(self._h, os.fsencode(path), fmt, fields, C.byref(n)))
        return n.value

    def partition_spmv(self, x, nparts):
        """y = K x formed through nparts row-block partitions (their halo
        exchange and local products) on this device."""
        neq, _, _ = self.sizes()
        y = np.zeros(neq)
        self._check(self._L.elx_partition_spmv(self._h, nparts, _ptr(_f64(x)), _ptr(y)))
        return y

    def partition_spmv_resident(self, nparts, reps=1):
        self._check(self._L.elx_partition_spmv_resident(self._h, nparts, reps))

    def partition_info(self, nparts, part):
        """(eq0, neq, nhalo) of one device partition (equations)."""
        a, b, h = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self._L.elx_partition_info(self._h, nparts, part, C.byref(a), C.byref(b),
                                               C.byref(h)))
        return a.value, b.value, h.value

    def state(self):
        """The resident (u (nnode, ndf), b0 (neq,))."""
        m = self.mesh
        neq, _, _ = self.sizes()
        u = np.zeros((m.nnode, m.ndf))
        b0 = np.zeros(neq)
        self._check(self._L.elx_get_state(self._h, _ptr(u), _ptr(b0)))
        return u, b0

    def assemble_resident(self):
        self._check(self._L.elx_assemble_resident(self._h))

    def solve_resident(self, solver=SOLVER_PCG, precision=PREC_FP64, tol=1e-11, maxit=10000,
                       ngram=50):
        info = Info()
        self._check(self._L.elx_solve_resident(self._h, solver, precision, tol, maxit, ngram,
                                               C.byref(info)))
        return info.as_dict()

    def update_resident(self):
        """u(id) = x on the device (update_mec without a host round trip)."""
        self._check(self._L.elx_update_resident(self._h))

    def spmv_resident(self, precision=PREC_FP64, reps=1):
        self._check(self._L.elx_spmv_resident(self._h, precision, reps))

    def solution(self):
        neq, _, _ = self.sizes()
        x = np.zeros(neq)
        self._check(self._L.elx_get_solution(self._h, x))
        return x

    def rhs(self):
        neq, _, _ = self.sizes()
        b = np.zeros(neq)
        self._check(self._L.elx_get_rhs(self._h, b))
        return b


# ---------------------------------------------------------------------------
# Reference-shaped entry points


def pform_mec(ctx: Context, u, b):
    """pform_mec(..., lhs=.true., rhs=.true., isw=2, ...) (Pform.f:1-11): forms
    K (kept on the device) and returns b - sum_e K_e u_e."""
    return ctx.assemble(u, b)


def solv(ctx: Context, b, tol=1e-11, maxit=10000, ngram=50, solver=SOLVER_PCG,
         precision=PREC_FP64):
    """solv(neq,nad,...,b,x,tol,maxit,ngram,...,solver,...) (Solv.f:13-15)."""
    return ctx.solve(b, solver=solver, precision=precision, tol=tol, maxit=maxit, ngram=ngram)


def fortran_e(x, w=15, d=5, e=0):
    """The device formatter's Ew.d (e = 0) / Ew.dEe fields of x (strings)."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    out = C.create_string_buffer(max(x.size * w, 1))
    st = load().elx_fortran_e(x.ctypes.data_as(_VP), x.size, w, d, e, C.cast(out, _VP))
    if st != OK:
        raise ElasticError(st, "elx_fortran_e failed")
    raw = out.raw[:x.size * w].decode()
    return [raw[i * w:(i + 1) * w] for i in range(x.size)]


def pload(mesh, id_eq):
    """pload_mec (Pload.f:2-58) for evaluated nodal forces: b0(id) = f for free
    dofs and u = f for prescribed ones.  Host-side, as in the reference."""
    id_eq = np.asarray(id_eq)
    neq = int(id_eq.max())
    b0 = np.zeros(neq)
    u = np.zeros_like(mesh.f)
    free = id_eq > 0
    b0[id_eq[free] - 1] = mesh.f[free]
    u[~free] = mesh.f[~free]
    return b0, u


def edge_loads(mesh, id_eq, b0):
    """2-D distributed edge loads of pform_mec isw=4 (Elmlib02.f:260-314 TRIA3,
    856-910 QUAD4): every loaded side adds traction * length / 2 to each of its
    two nodes.  Host-side, as in the reference."""
    if mesh.eload is None:
        return b0
    b0 = b0.copy()
    tri = {1: (0, 1), 2: (1, 2), 3: (2, 0)}
    quad = {1: (0, 1), 2: (1, 2), 3: (2, 3), 4: (3, 0)}
    for el in np.nonzero(mesh.eload.sum(axis=1) > 0)[0]:
        iel = int(mesh.ie[mesh.ix[el, mesh.nen] - 1])
        sides = tri if iel in (2, 3) else quad
        p = np.zeros((4, 2))
        for sd, (a, b) in sides.items():
            lc = int(mesh.eload[el, sd - 1])
            if lc <= 0:
                continue
            na, nb = mesh.ix[el, a] - 1, mesh.ix[el, b] - 1
            dx = mesh.x[nb] - mesh.x[na]
            det = dx[0] * dx[0] + dx[1] * dx[1]
            if det <= 0.0:
                raise ElasticError(ERR_BAD_DET, f"zero-length loaded side in element {el + 1}")
            wt1 = 0.5 * np.sqrt(det)
            ff = mesh.loadvec[lc - 1]
            p[a] -= ff * wt1
            p[b] -= ff * wt1
        for a in range(len(sides)):
            no = mesh.ix[el, a] - 1
            for d in range(2):
                k = id_eq[no, d]
                if k > 0:
                    b0[k - 1] -= p[a, d]
    return b0


def solvm(mesh, tol=1e-11, maxit=10000, maxnlit=2, nl_tol=1e-4, solver=SOLVER_PCG,
          precision=PREC_FP64, reorder=True, ctx: Context | None = None):
    """The reference driver's solvm macro (Main.f:718-849) on the library: loads,
    then up to maxnlit passes of assemble -> residual test -> solve -> update.
    Returns (u, info, ctx)."""
    own = ctx is None
    ctx = ctx or Context()
    ctx.set_mesh(mesh)
    ctx.build_structure(reorder)
    st = ctx.structure()
    b0, u = pload(mesh, st.id)
    b0 = edge_loads(mesh, st.id, b0)
    resid0 = 0.0
    info = None
    for i in range(1, maxnlit + 1):
        b = ctx.assemble(u, b0)
        resid = float(np.sqrt(b @ b))
        if i == 1:
            resid0 = max(resid0, resid)
        if resid0 > 0 and resid / resid0 < nl_tol:
            break
        x, info = ctx.solve(b, solver=solver, precision=precision, tol=tol, maxit=maxit)
        u = ctx.update(x, u)
    if own:
        return u, info, ctx
    return u, info, ctx


class Server:
    """Solve server (elx_server_*): submit meshes with load cases, collect
    nodal displacements; requests are batched continuously on the GPU."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, prep_threads: int = 4,
                 poll_steps: int = 8, max_slots: int = 4096, large_dofs: int = 0,
                 large_mode: int = 0, large_workers: int = 0):
        """large_dofs: requests with at least this many equations are solved
        whole by the block PCG (0: library default 100000); large_mode 0 auto
        (mixed in 3-D, FP64 in 2-D), 1 FP64, 2 mixed, -1 pack everything."""
        self._L = load()
        self._h = _VP()
        o = ServerOpts(device, prep_threads, hbm_budget, poll_steps, max_slots, large_dofs,
                       large_mode, large_workers)
        st = self._L.elx_server_create(C.byref(self._h), C.byref(o))
        if st != OK:
            raise ElasticError(st, "server creation failed")
        self._shapes = {}

    def submit(self, mesh, F, tol=1e-8, maxit=20000) -> int:
        """F: nodal forces (nnode, ndf) or (nrhs, nnode, ndf).  Returns a ticket."""
        F = np.ascontiguousarray(F, dtype=np.float64)
        if F.ndim == 2:
            F = F[None]
        e = _f64(mesh.e)
        t = C.c_int64(0)
        st = self._L.elx_server_submit(self._h, mesh.ndm, mesh.ndf, mesh.nen, mesh.numel,
                                       mesh.nnode, _i32(mesh.ix), _f64(mesh.x), _i32(mesh.ie),
                                       e, e.shape[1], e.shape[0], _i32(mesh.id), F.shape[0],
                                       F, tol, maxit, C.byref(t))
        if st != OK:
            raise ElasticError(st, "submit failed")
        self._shapes[t.value] = F.shape
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        """(U (nrhs, nnode, ndf), infos, latency_s, status); raises on timeout."""
        shape = self._shapes[ticket]
        U = np.zeros(shape)
        infos = (Info * shape[0])()
        lat = C.c_double(0)
        st = self._L.elx_server_wait(self._h, ticket, timeout, U.ctypes.data_as(_VP),
                                     C.cast(infos, _VP), C.byref(lat))
        if st == ERR_TIMEOUT:
            raise ElasticError(st, "request not done yet")
        del self._shapes[ticket]
        return U, [i.as_dict() for i in infos], lat.value, st

    def stats(self) -> dict:
        s = ServerStats()
        self._L.elx_server_get_stats(self._h, C.byref(s))
        return s.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            self._L.elx_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
