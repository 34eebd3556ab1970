"""CPU oracle for the Elastic linear-elasticity solve path.

TEST INFRASTRUCTURE ONLY: the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use this module to check (or to time, as the
reference's own CPU path) the CUDA library.  The product package
``elastic_gb300`` never imports it.

The numerics live in ``elx_oracle.c`` (a restatement of the reference's
Fortran routines, each citing its file:line); this module is a thin ctypes
wrapper that also replays the reference driver's ``solvm`` sequence
(mef/src/Main.f:718-849).
"""
from __future__ import annotations

import ctypes as C
import fcntl
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

STATUS = {0: "ok", 1: "zero diagonal", 2: "no convergence", 3: "bad determinant",
          4: "out of memory", 6: "bad argument", 7: "bad element type"}


class OracleError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__(f"oracle: {STATUS.get(code, code)} {what}".strip())
        self.code = code


class Info(C.Structure):
    _fields_ = [("iters", C.c_int), ("status", C.c_int), ("xkx", C.c_double),
                ("norm_x", C.c_double), ("norm_r", C.c_double),
                ("norm_m_r", C.c_double), ("conv", C.c_double),
                ("seconds", C.c_double), ("mflops", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build():
    """Compile oracle/_build/liboracle.so with the committed Makefile (under
    an exclusive lock: test workers may ask at once; the Makefile links to a
    temporary name and renames it into place)."""
    os.makedirs(os.path.join(_HERE, "_build"), exist_ok=True)
    with open(os.path.join(_HERE, "_build", ".lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO) or (
                os.path.getmtime(_SO) < os.path.getmtime(os.path.join(_HERE, "elx_oracle.c"))):
            build()
        L = C.CDLL(_SO)
        L.orc_graph.restype = C.c_int
        L.orc_graph.argtypes = [I32P, C.c_int, C.c_int, C.c_int, I32P, I32P, C.c_int]
        L.orc_reord.argtypes = [I32P, C.c_int, C.c_int, C.c_int, I32P]
        L.orc_numeq.argtypes = [I32P, I32P, C.c_int, C.c_int]
        L.orc_csr_ia.restype = C.c_longlong
        L.orc_csr_ia.argtypes = [I32P, I32P, I32P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, I32P]
        L.orc_csr_ja.argtypes = [I32P, I32P, I32P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, I32P, I32P]
        L.orc_element_stiffness.argtypes = [C.c_int, F64P, F64P, C.c_int, F64P]
        L.orc_pform_k.argtypes = [I32P, I32P, F64P, C.c_int, F64P, I32P, I32P, I32P, F64P, F64P,
                                  F64P, F64P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_int, C.c_longlong, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_pform_edge_loads.argtypes = [I32P, I32P, F64P, I32P, I32P, F64P, F64P, C.c_int,
                                           C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_pload.argtypes = [I32P, F64P, F64P, F64P, C.c_int, C.c_int]
        L.orc_tform.argtypes = [I32P, I32P, F64P, C.c_int, F64P, F64P, C.c_void_p, C.c_int,
                                C.c_int, C.c_int, C.c_int, C.c_int, F64P, I32P,
                                C.POINTER(C.c_int)]
        L.orc_update.argtypes = [I32P, F64P, F64P, C.c_int, C.c_int]
        L.orc_write_mesh_res.argtypes = [C.c_char_p, C.c_int, I32P, I32P, F64P, C.c_void_p,
                                         C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_int]
        L.orc_fortran_e.argtypes = [F64P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p]
        L.orc_csr_right.argtypes = [I32P, I32P, I32P, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.orc_matvec_csrcrsym1.argtypes = [C.c_int, I32P, I32P, I32P, I32P, F64P, F64P, F64P,
                                           F64P, F64P]
        L.orc_matvec_csrcsym1.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P, F64P]
        L.orc_dot.restype = C.c_double
        L.orc_dot.argtypes = [F64P, F64P, C.c_int]
        L.orc_flop_cg.restype = C.c_double
        L.orc_flop_cg.argtypes = [C.c_int, C.c_longlong, C.c_int]
        L.orc_pre_diag.argtypes = [F64P, F64P, C.c_int]
        sol = [C.c_int, C.c_longlong, I32P, I32P, F64P, F64P, F64P, F64P]
        L.orc_pcg.argtypes = sol + [C.c_double, C.c_int, C.POINTER(Info)]
        L.orc_pbicgstab.argtypes = sol + [C.c_double, C.c_int, C.POINTER(Info)]
        L.orc_bicgstab.argtypes = sol + [C.c_double, C.c_int, C.POINTER(Info)]
        L.orc_gmres.argtypes = sol + [C.c_int, C.c_double, C.c_int, C.POINTER(Info)]
        L.orc_pcg_omp.argtypes = sol + [C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(Info)]
        L.orc_matvec_csrcsym_omp.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P, F64P, C.c_int,
                                             C.c_int, C.POINTER(C.c_double)]
        L.orc_max_threads.restype = C.c_int
        L.orc_colormsh.argtypes = [I32P, C.c_int, C.c_int, C.c_int, C.c_int, I32P, I32P, C.c_int]
        L.orc_pform_k_omp.argtypes = [I32P, I32P, F64P, C.c_int, F64P, I32P, I32P, I32P, F64P,
                                      F64P, F64P, F64P, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int, C.c_int, C.c_longlong, I32P, I32P, C.c_int,
                                      C.c_int, C.POINTER(C.c_int)]
        _lib = L
    return _lib


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class Structure:
    """Equation numbering and CSRC pattern, 1-based as in the reference."""
    perm: np.ndarray   # (nnode,) old node at new position k (Reord.f)
    id: np.ndarray     # (nnode, ndf) equation numbers, 0 = constrained
    neq: int
    nad: int
    ia: np.ndarray     # (neq+1,) 1-based
    ja: np.ndarray     # (nad,) 1-based, ascending per row


def graph(mesh):
    L = lib()
    ix = _i32(mesh.ix)
    ip = np.zeros(mesh.nnode + 1, np.int32)
    cap = mesh.numel * mesh.nen * (mesh.nen - 1) + 1
    adj = np.zeros(cap, np.int32)
    n = L.orc_graph(ix, mesh.nnode, mesh.numel, mesh.nen, ip, adj, cap)
    if n < 0:
        raise OracleError(-n, "graph")
    return ip, adj[:n].copy()


def structure(mesh, reorder=True) -> Structure:
    """reord (Reord.f:1) + numeq (Numeq.f:139) + csrstruct lower-only (Csr.f:13)."""
    L = lib()
    ix = _i32(mesh.ix)
    if reorder:
        perm = np.zeros(mesh.nnode, np.int32)
        st = L.orc_reord(ix, mesh.nnode, mesh.numel, mesh.nen, perm)
        if st:
            raise OracleError(st, "reord")
    else:
        perm = np.arange(1, mesh.nnode + 1, dtype=np.int32)
    idm = _i32(mesh.id).copy()
    neq = L.orc_numeq(idm, perm, mesh.nnode, mesh.ndf)
    ia = np.zeros(neq + 1, np.int32)
    nad = L.orc_csr_ia(idm, perm, ix, mesh.nnode, mesh.numel, mesh.nen, mesh.ndf, neq, ia)
    if nad < 0:
        raise OracleError(-nad, "csria")
    ja = np.zeros(max(nad, 1), np.int32)
    st = L.orc_csr_ja(idm, perm, ix, mesh.nnode, mesh.numel, mesh.nen, mesh.ndf, neq, ia, ja)
    if st:
        raise OracleError(st, "csrja")
    return Structure(perm=perm, id=idm, neq=int(neq), nad=int(nad), ia=ia, ja=ja[:nad])


def element_stiffness(iel, e, xl):
    """One element matrix s(nst,nst) as a numpy (nst, nst) array s[row, col]."""
    L = lib()
    nst = {2: 6, 3: 6, 4: 8, 5: 8, 6: 12, 7: 24}[iel]
    ndm = 2 if iel <= 5 else 3
    s = np.zeros(nst * nst)
    ev = np.zeros(15)
    ev[:len(e)] = e
    st = L.orc_element_stiffness(iel, ev, _f64(np.asarray(xl).reshape(-1)), ndm, s)
    if st:
        raise OracleError(st, "element")
    return s.reshape(nst, nst).T.copy()  # column-major -> [row, col]


def assemble(mesh, s: Structure, u=None, b0=None, lhs=True, rhs=True):
    """pform_mec(isw=2) (Pform.f:1-254 + Assbly.f:66-146): returns (ad, al, b)
    with b = b0 - K u (rows of free dofs)."""
    L = lib()
    ad = np.zeros(s.neq)
    al = np.zeros(max(s.nad, 1))
    b = _f64(b0).copy() if b0 is not None else np.zeros(s.neq)
    u = _f64(u) if u is not None else np.zeros((mesh.nnode, mesh.ndf))
    bad = C.c_int(0)
    st = L.orc_pform_k(_i32(mesh.ix), _i32(mesh.ie), _f64(mesh.e), mesh.e.shape[1],
                       _f64(mesh.x), s.id, s.ia, _i32(s.ja) if s.nad else np.zeros(1, np.int32),
                       al, ad, b, u, mesh.numel, mesh.nen, mesh.nen, mesh.ndf, mesh.ndm,
                       s.neq, s.nad, int(lhs), int(rhs), C.byref(bad))
    if st:
        raise OracleError(st, f"element {bad.value}")
    return ad, al[:s.nad], b


def tform(mesh, u, tx0=None):
    """tform_mec (Pform.f:258-421) with the elements' isw = 3: nodal stresses
    t (nnode, ntn), averaged over each node's elements, + tx0."""
    L = lib()
    ntn = 4 if mesh.ndm == 2 else 6
    t = np.zeros((mesh.nnode, ntn))
    ic = np.zeros(mesh.nnode, np.int32)
    bad = C.c_int(0)
    tx0p = None if tx0 is None else _f64(tx0).ctypes.data_as(C.c_void_p)
    st = L.orc_tform(_i32(mesh.ix), _i32(mesh.ie), _f64(mesh.e), mesh.e.shape[1], _f64(mesh.x),
                     _f64(u), tx0p, mesh.nnode, mesh.numel, mesh.nen, mesh.ndm, mesh.ndf, t, ic,
                     C.byref(bad))
    if st:
        raise OracleError(st, f"element {bad.value}")
    return t


def write_mesh_res(path, mesh, u=None, t=None, fmt=0):
    """write_mesh_res_mec (Write_vtk.f:742-985): the result file at `path`,
    fmt 0 the XML VTU ASCII file, 1 the legacy binary VTK file; u (nnode,
    ndf) -> "desloc", t (nnode, ntn) -> "stress"."""
    ntn = 4 if mesh.ndm == 2 else 6
    up = None if u is None else _f64(u).ctypes.data_as(C.c_void_p)
    tp = None if t is None else _f64(t).ctypes.data_as(C.c_void_p)
    st = lib().orc_write_mesh_res(os.fsencode(path), fmt, _i32(mesh.ix), _i32(mesh.ie),
                                  _f64(mesh.x), up, tp, mesh.nnode, mesh.numel, mesh.nen,
                                  mesh.ndm, mesh.ndf, ntn)
    if st:
        raise OracleError(st, "write_mesh_res")


def fortran_e(x, w=15, d=5, e=0):
    """Fortran Ew.d (e = 0) / Ew.dEe fields of x as gfortran prints them."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    out = C.create_string_buffer(max(x.size * w, 1))
    lib().orc_fortran_e(x, x.size, w, d, e, out)
    raw = out.raw[:x.size * w].decode()
    return [raw[i * w:(i + 1) * w] for i in range(x.size)]


def csr_right(mesh, local_id, perm, neq):
    """csrstruct with lower = right = .true. (Csr.f:13-305) on a partition's
    local equation numbers local_id (nnode, ndf; owned 1..neq, halo > neq,
    0 elsewhere): (ia, ja, ia1, ja1), 1-based, both parts sorted per row."""
    L = lib()
    nad, nad1 = C.c_longlong(0), C.c_longlong(0)
    lid = _i32(local_id)
    st = L.orc_csr_right(lid, _i32(perm), _i32(mesh.ix), mesh.nnode, mesh.numel, mesh.nen,
                         mesh.ndf, neq, None, None, C.byref(nad), C.byref(nad1))
    if st:
        raise OracleError(st, "csr_right")
    ia = np.zeros(2 * neq + 2, np.int32)
    ja = np.zeros(max(nad.value + nad1.value, 1), np.int32)
    st = L.orc_csr_right(lid, _i32(perm), _i32(mesh.ix), mesh.nnode, mesh.numel, mesh.nen,
                         mesh.ndf, neq, ia.ctypes.data_as(C.c_void_p),
                         ja.ctypes.data_as(C.c_void_p), C.byref(nad), C.byref(nad1))
    if st:
        raise OracleError(st, "csr_right")
    n = nad.value
    return ia[:neq + 1], ja[:n], ia[neq + 1:], ja[n:n + nad1.value]


def matvec_csrcrsym1(neq, ia, ja, ia1, ja1, ad, al, ar, x):
    """matvec_csrcrsym1 (Matvec.f:1090-1191): y(neq) on a partition, x = the
    owned then the halo values."""
    y = np.zeros(neq)
    z1 = lambda a, t: a if len(a) else np.zeros(1, t)
    lib().orc_matvec_csrcrsym1(neq, _i32(ia), z1(_i32(ja), np.int32), _i32(ia1),
                               z1(_i32(ja1), np.int32), _f64(ad), z1(_f64(al), np.float64),
                               z1(_f64(ar), np.float64), _f64(x), y)
    return y


def colormsh(mesh):
    """coloredmesh with omp_elmt (Colormsh.f:9-308): (elcolor, colorg)."""
    elcolor = np.zeros(mesh.numel, np.int32)
    colorg = np.zeros(2 * 200, np.int32)
    nc = lib().orc_colormsh(_i32(mesh.ix), mesh.nnode, mesh.numel, mesh.nen, mesh.nen,
                            elcolor, colorg, 200)
    if nc < 0:
        raise OracleError(-nc, "colormsh")
    return elcolor, colorg[:2 * nc].copy()


def assemble_omp(mesh, s: Structure, u=None, b0=None, nthreads=None, colors=None):
    """pform_mec(isw=2) with the OpenMP colour loop (Pform.f:108-183)."""
    L = lib()
    nth = nthreads or L.orc_max_threads()
    elcolor, colorg = colors if colors is not None else colormsh(mesh)
    ad = np.zeros(s.neq)
    al = np.zeros(max(s.nad, 1))
    b = _f64(b0).copy() if b0 is not None else np.zeros(s.neq)
    u = _f64(u) if u is not None else np.zeros((mesh.nnode, mesh.ndf))
    bad = C.c_int(0)
    st = L.orc_pform_k_omp(_i32(mesh.ix), _i32(mesh.ie), _f64(mesh.e), mesh.e.shape[1],
                           _f64(mesh.x), s.id, s.ia, _i32(s.ja), al, ad, b, u, mesh.numel,
                           mesh.nen, mesh.nen, mesh.ndf, mesh.ndm, s.neq, s.nad, elcolor,
                           colorg, colorg.shape[0] // 2, nth, C.byref(bad))
    if st:
        raise OracleError(st, f"element {bad.value}")
    return ad, al[:s.nad], b


def loads(mesh, s: Structure):
    """pload_mec (Pload.f:2-58) then pform_mec isw=4 edge loads: (b0, u)."""
    L = lib()
    b0 = np.zeros(s.neq)
    u = np.zeros((mesh.nnode, mesh.ndf))
    L.orc_pload(s.id, _f64(mesh.f), u, b0, mesh.nnode, mesh.ndf)
    if mesh.eload is not None:
        bad = C.c_int(0)
        st = L.orc_pform_edge_loads(_i32(mesh.ix), _i32(mesh.ie), _f64(mesh.x), s.id,
                                    _i32(mesh.eload), _f64(mesh.loadvec), b0, mesh.numel,
                                    mesh.nen, mesh.ndf, mesh.ndm, s.neq, C.byref(bad))
        if st:
            raise OracleError(st, f"edge load element {bad.value}")
    return b0, u


def matvec(s: Structure, ad, al, x):
    """matvec_csrcsym1 (Matvec.f:528-621)."""
    y = np.zeros(s.neq)
    lib().orc_matvec_csrcsym1(s.neq, s.ia, _i32(s.ja) if s.nad else np.zeros(1, np.int32),
                              _f64(ad), _f64(al) if s.nad else np.zeros(1), _f64(x), y)
    return y


def _solve(fn, s, ad, al, b, *extra):
    x = np.zeros(s.neq)
    info = Info()
    ja = _i32(s.ja) if s.nad else np.zeros(1, np.int32)
    alv = _f64(al) if s.nad else np.zeros(1)
    st = fn(s.neq, s.nad, s.ia, ja, _f64(ad), alv, _f64(b), x, *extra, C.byref(info))
    return x, info.as_dict()


def pcg(s, ad, al, b, tol=1e-11, maxit=10000):
    """pcg (Iters.f:252-524) with the Jacobi preconditioner of Solv.f:65-69."""
    return _solve(lib().orc_pcg, s, ad, al, b, tol, maxit)


def pcg_omp(s, ad, al, b, tol=1e-11, maxit=10000, nthreads=None, stop_at_maxit=False):
    """pcg_omp (Iters_omp.f:17-334) with matvec_csrcsym_omp."""
    nth = nthreads or lib().orc_max_threads()
    return _solve(lib().orc_pcg_omp, s, ad, al, b, tol, maxit, nth, int(stop_at_maxit))


def pbicgstab(s, ad, al, b, tol=1e-11, maxit=10000):
    """pbicgstab (Iters.f:1079-1349)."""
    return _solve(lib().orc_pbicgstab, s, ad, al, b, tol, maxit)


def flop_cg(neq, nad, iters):
    """flop_cg (Matvec.f:1499-1531): the PCG's floating-point operations."""
    return lib().orc_flop_cg(int(neq), int(nad), int(iters))


def bicgstab(s, ad, al, b, tol=1e-11, maxit=10000):
    """bicgstab (Iters.f:812-1075): no preconditioner, beta from (r, b)."""
    return _solve(lib().orc_bicgstab, s, ad, al, b, tol, maxit)


def gmres(s, ad, al, b, k=50, tol=1e-11, maxit=10000):
    """gmres (Iters.f:528-808); maxit counts restart cycles."""
    return _solve(lib().orc_gmres, s, ad, al, b, k, tol, maxit)


def matvec_omp(s, ad, al, x, nthreads=None, reps=1):
    """matvec_csrcsym_omp (Matvec_omp.f:150-245); returns (y, seconds)."""
    nth = nthreads or lib().orc_max_threads()
    y = np.zeros(s.neq)
    sec = C.c_double(0)
    st = lib().orc_matvec_csrcsym_omp(s.neq, s.ia, _i32(s.ja), _f64(ad), _f64(al), _f64(x), y,
                                      nth, reps, C.byref(sec))
    if st:
        raise OracleError(st, "matvec_omp")
    return y, sec.value


def update(s: Structure, xsol, u):
    """update_mec (Predict.f:183-209)."""
    u = _f64(u).copy()
    lib().orc_update(s.id, _f64(xsol), u, u.shape[0], u.shape[1])
    return u


def solvm(mesh, tol=1e-11, maxit=10000, maxnlit=2, nl_tol=1e-4, solver="pcg",
          reorder=True, s=None):
    """Replay of the reference driver's solvm macro (Main.f:718-849) for a
    linear problem: loads, then up to maxnlit passes of assemble -> residual
    test -> solve -> update.  Returns (u, info of the solve, structure, ad, al)."""
    s = s or structure(mesh, reorder)
    b0, u = loads(mesh, s)
    resid0 = 0.0
    info = None
    ad = al = None
    for i in range(1, maxnlit + 1):
        ad, al, b = assemble(mesh, s, u, b0)
        resid = float(np.sqrt(lib().orc_dot(b, b, s.neq)))
        if i == 1:
            resid0 = max(resid0, resid)
        if resid0 > 0 and resid / resid0 < nl_tol:
            break
        if solver == "pcg":
            x, info = pcg(s, ad, al, b, tol, maxit)
        elif solver == "bicgstab":
            x, info = pbicgstab(s, ad, al, b, tol, maxit)
        elif solver == "gmres":
            x, info = gmres(s, ad, al, b, 50, tol, maxit)
        else:
            raise ValueError(solver)
        if info["status"] != 0:
            raise OracleError(info["status"], "solve")
        u = update(s, x, u)
    return u, info, s, ad, al
