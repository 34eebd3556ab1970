"""Edge cases of the solve path on the GPU: the smallest meshes (one element
of each type), a zero load (x = 0 exactly, where the reference's PCG
divides 0 by 0), no free equation, maxit = 0, a mesh with every node fixed
but one, and a served request whose load cases are all zero."""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rel_inf

pytestmark = pytest.mark.gpu

ONE = {
    "hexa8": lambda: M.box_hexa8(1, 1, 1),
    "tetra4": lambda: M.box_tetra4(1, 1, 1),
    "quad4": lambda: M.box2d(1, 1, etype=M.QUAD4_STRESS),
    "tria3": lambda: M.box2d(1, 1, etype=M.TRIA3_STRAIN),
}


@pytest.mark.parametrize("name", sorted(ONE))
def test_single_element_meshes(gpu_ctx, name):
    m = ONE[name]()
    m.f = np.random.default_rng(1).standard_normal(m.f.shape) * (m.id == 0)
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    s = O.structure(m, True)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    x_o, _ = O.pcg(s, ad, al, b, tol=1e-12, maxit=1000)
    b_g = gpu_ctx.assemble(u0, b0)
    assert rel_inf(b, b_g) <= 1e-13
    for prec in (E.PREC_FP64, E.PREC_MIXED):
        x_g, info = gpu_ctx.solve(b_g, tol=1e-12, maxit=1000, precision=prec)
        assert info["status"] == 0
        assert rel_inf(x_o, x_g) <= (1e-10 if prec == E.PREC_FP64 else 1e-6)


@pytest.mark.parametrize("solver,prec", [(E.SOLVER_PCG, E.PREC_FP64),
                                         (E.SOLVER_PCG, E.PREC_MIXED),
                                         (E.SOLVER_BICGSTAB, E.PREC_FP64),
                                         (E.SOLVER_GMRES, E.PREC_FP64)])
def test_zero_load_gives_zero_displacement(gpu_ctx, solver, prec):
    m = M.box_hexa8(4, 3, 3)
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    neq = gpu_ctx.sizes()[0]
    gpu_ctx.assemble(None, None)
    x, info = gpu_ctx.solve(np.zeros(neq), solver=solver, precision=prec, tol=1e-10)
    assert info["status"] == 0 and info["iters"] == 0
    assert np.array_equal(x, np.zeros(neq))


def test_zero_load_cases_in_a_block(gpu_ctx):
    m = M.box_hexa8(5, 4, 3)
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    neq = gpu_ctx.sizes()[0]
    gpu_ctx.assemble(None, None)
    B = np.random.default_rng(2).standard_normal((neq, 4))
    B[:, 1] = 0.0
    X, infos = gpu_ctx.solve_block(B, precision=E.PREC_FP64, tol=1e-10, width=4)
    assert np.array_equal(X[:, 1], np.zeros(neq)) and infos[1]["iters"] == 0
    x0, _ = gpu_ctx.solve(B[:, 0], tol=1e-10)
    assert rel_inf(x0, X[:, 0]) <= 1e-8


def test_no_free_equation_is_refused(gpu_ctx):
    m = M.box_hexa8(1, 1, 1)
    m.id[:] = 1  # every dof prescribed
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.set_mesh(m)
        gpu_ctx.build_structure(True)
    assert e.value.code == E.ERR_ARG


def test_one_free_node(gpu_ctx):
    m = M.box_hexa8(1, 1, 1)
    m.id[:] = 1
    m.id[-1] = 0  # only the last node free: a 3x3 system
    m.f[:] = 0.0
    m.f[-1] = [0.1, -0.2, 0.3]
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    s = O.structure(m, True)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    K = np.diag(ad)
    for r in range(3):
        for k in range(s.ia[r] - 1, s.ia[r + 1] - 1):
            c = s.ja[k] - 1
            K[r, c] = K[c, r] = al[k]
    x_g, info = gpu_ctx.solve(gpu_ctx.assemble(u0, b0), tol=1e-14, maxit=10)
    assert info["status"] == 0 and info["iters"] <= 3
    assert rel_inf(np.linalg.solve(K, b), x_g) <= 1e-12


def test_maxit_zero_reports_no_convergence(gpu_ctx):
    m = M.box_hexa8(3, 3, 3)
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    b = gpu_ctx.assemble(None, np.ones(gpu_ctx.sizes()[0]))
    x, info = gpu_ctx.solve(b, tol=1e-10, maxit=0, raise_on_error=False)
    assert info["status"] == E.ERR_NO_CONVERGENCE and info["iters"] == 0
    assert np.array_equal(x, np.zeros_like(x))


def test_served_zero_request(built_lib):
    m = M.box_hexa8(4, 4, 3)
    F = np.zeros((2,) + m.f.shape)
    with E.Server(device=0) as srv:
        U, infos, _, status = srv.wait(srv.submit(m, F, tol=1e-10), timeout=300)
        assert status == 0 and all(i["iters"] == 0 for i in infos)
        assert np.array_equal(U, np.zeros_like(U))
