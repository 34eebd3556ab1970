"""GPU stress recovery (elx_stress = tform_mec, Pform.f:258-421, with the
elements' isw = 3) against the oracle's restatement: nodal stresses within
1e-12 of the largest, for every element type, with initial stresses, after a
real solve, and the reference's non-positive-Jacobian error."""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M

pytestmark = pytest.mark.gpu

MESHES = {
    "tria3_strain": lambda: M.box2d(12, 9, 2.0, 1.0, etype=M.TRIA3_STRAIN, E=3.0, nu=0.25),
    "tria3_stress": lambda: M.box2d(12, 9, 2.0, 1.0, etype=M.TRIA3_STRESS, E=3.0, nu=0.25),
    "quad4_strain": lambda: M.box2d(16, 8, 2.0, 1.0, etype=M.QUAD4_STRAIN),
    "quad4_stress": lambda: M.cantilever_quad4_64x16(),
    "tetra4": lambda: M.box_tetra4(7, 6, 5, jitter=0.2, lognormal_E=True, seed=4),
    "hexa8": lambda: M.box_hexa8(9, 8, 7, jitter=0.2, seed=5),
}


def _rel(ref, got):
    return np.abs(ref - got).max() / np.abs(ref).max()


@pytest.mark.parametrize("name", sorted(MESHES))
def test_stress_matches_oracle(gpu_ctx, name):
    m = MESHES[name]()
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    rng = np.random.default_rng(8)
    u = rng.standard_normal((m.nnode, m.ndf)) * 1e-3
    t_o = O.tform(m, u)
    t_g = gpu_ctx.stress(u)
    assert _rel(t_o, t_g) <= 1e-12
    tx0 = rng.standard_normal(t_o.shape)
    assert _rel(O.tform(m, u, tx0), gpu_ctx.stress(u, tx0)) <= 1e-12


@pytest.mark.parametrize("name", ["quad4_stress", "hexa8"])
def test_stress_after_solve(gpu_ctx, name):
    m = MESHES[name]()
    u, info, ctx = E.solvm(m, tol=1e-11, ctx=gpu_ctx)
    t_g = ctx.stress(u)
    assert _rel(O.tform(m, u), t_g) <= 1e-12
    assert np.isfinite(t_g).all()


def test_stress_bad_jacobian(gpu_ctx):
    m = M.box_hexa8(3, 3, 3)
    m.ix[4, :8] = m.ix[4, [4, 5, 6, 7, 0, 1, 2, 3]]  # one element turned inside out
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.stress(np.zeros((m.nnode, 3)))
    assert e.value.code == E.ERR_BAD_DET


def test_resident_pass_matches_host_pass(gpu_ctx):
    """assemble -> solve -> update -> stresses on the device only, against
    the same pass through host buffers."""
    m = MESHES["hexa8"]()
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    st = gpu_ctx.structure()
    b0, u0 = E.pload(m, st.id)
    b = gpu_ctx.assemble(u0, b0)
    x, _ = gpu_ctx.solve(b, tol=1e-11)
    u = gpu_ctx.update(x, u0)
    t_host = gpu_ctx.stress(u)
    gpu_ctx.set_state(u0, b0)
    gpu_ctx.assemble_resident()
    gpu_ctx.solve_resident(tol=1e-11)
    gpu_ctx.update_resident()
    t_dev = gpu_ctx.stress(None)
    assert np.array_equal(t_dev, t_host)
