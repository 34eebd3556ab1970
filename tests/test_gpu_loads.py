"""Device loads (elx_set_loads = pload_mec, Pload.f:2-58, and the 2-D edge
loads of pform_mec isw = 4, Elmlib02.f:260-314 / 856-910) against the
oracle's restatement (orc_pload + orc_pform_edge_loads): b0 and u bitwise
equal; errors as the reference's; and the whole load -> assemble -> solve ->
update -> stress pass on the device, bitwise equal to the pass through host
buffers."""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def _two_loads(m, rng):
    """Side loads with two load numbers on several sides (corner elements
    get two loaded sides), plus random nodal loads on free and fixed dofs."""
    m.loadvec = np.array([[0.3, -1.0], [-0.7, 0.25]])
    eload = np.zeros((m.numel, 7), np.int32)
    nside = 3 if m.ie[0] in (M.TRIA3_STRAIN, M.TRIA3_STRESS) else 4
    for el in rng.choice(m.numel, size=max(1, m.numel // 5), replace=False):
        sides = rng.choice(nside, size=rng.integers(1, 3), replace=False)
        eload[el, sides] = rng.integers(1, 3, size=len(sides))
    m.eload = eload
    m.f = rng.standard_normal(m.f.shape)
    return m


MESHES = {
    "cantilever": lambda rng: M.cantilever_quad4_64x16(),
    "tria3_top": lambda rng: M.box2d(10, 7, 2.0, 1.0, etype=M.TRIA3_STRESS,
                                     traction=(0.5, -2.0), traction_side="top"),
    "quad4_random": lambda rng: _two_loads(M.box2d(9, 6, 2.0, 1.5, etype=M.QUAD4_STRAIN), rng),
    "tria3_random": lambda rng: _two_loads(M.box2d(8, 8, 1.0, 1.0, etype=M.TRIA3_STRAIN), rng),
}


def _setup(ctx, m):
    ctx.set_mesh(m)
    ctx.build_structure(True)
    return O.structure(m, True)


@pytest.mark.parametrize("name", sorted(MESHES))
def test_device_loads_match_oracle_bitwise(gpu_ctx, name):
    m = MESHES[name](np.random.default_rng(11))
    s = _setup(gpu_ctx, m)
    b0_o, u_o = O.loads(m, s)
    gpu_ctx.set_state(None, None)
    gpu_ctx.set_loads(m.f, m.eload, m.loadvec)
    u_g, b0_g = gpu_ctx.state()
    assert np.array_equal(b0_g, b0_o)
    assert np.array_equal(u_g, u_o)
    # the host-side mirror gives the same bits
    st = gpu_ctx.structure()
    b0_h, _ = E.pload(m, st.id)
    assert np.array_equal(E.edge_loads(m, st.id, b0_h), b0_g)


def test_free_dofs_of_u_keep_their_values(gpu_ctx):
    m = MESHES["quad4_random"](np.random.default_rng(3))
    _setup(gpu_ctx, m)
    u_prev = np.random.default_rng(4).standard_normal((m.nnode, m.ndf))
    gpu_ctx.set_state(u_prev, None)
    gpu_ctx.set_loads(m.f)
    u_g, _ = gpu_ctx.state()
    st = gpu_ctx.structure()
    free = st.id > 0
    assert np.array_equal(u_g[free], u_prev[free])
    assert np.array_equal(u_g[~free], m.f[~free])


def test_load_errors(gpu_ctx):
    m = MESHES["quad4_random"](np.random.default_rng(5))
    _setup(gpu_ctx, m)
    bad = m.eload.copy()
    bad[0, 0] = 3  # only two loads defined
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.set_loads(m.f, bad, m.loadvec)
    assert e.value.code == E.ERR_ARG
    side5 = np.zeros_like(m.eload)
    side5[0, 4] = 1  # a QUAD4 has four sides
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.set_loads(m.f, side5, m.loadvec)
    assert e.value.code == E.ERR_ARG
    # a loaded side of zero length
    m2 = M.box2d(4, 3, 1.0, 1.0, etype=M.QUAD4_STRESS, traction=(0.0, -1.0),
                 traction_side="right")
    _setup(gpu_ctx, m2)
    el = int(np.nonzero(m2.eload[:, 1])[0][0])
    a, b = m2.ix[el, 1] - 1, m2.ix[el, 2] - 1
    m2.x[b] = m2.x[a]
    gpu_ctx.set_mesh(m2)
    gpu_ctx.build_structure(True)
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.set_loads(m2.f, m2.eload, m2.loadvec)
    assert e.value.code == E.ERR_BAD_DET
    # 3-D meshes have no distributed edge loads in the reference
    m3 = M.box_hexa8(3, 3, 3)
    _setup(gpu_ctx, m3)
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.set_loads(m3.f, np.zeros((m3.numel, 7), np.int32), np.zeros((1, 2)))
    assert e.value.code == E.ERR_ARG


@pytest.mark.parametrize("name", ["cantilever", "tria3_random"])
def test_device_pass_matches_host_pass(gpu_ctx, name):
    """loads -> assemble -> solve -> update -> stresses with nothing but the
    loads' inputs crossing to the device, against the host-buffer pass."""
    m = MESHES[name](np.random.default_rng(13))
    _setup(gpu_ctx, m)
    st = gpu_ctx.structure()
    b0, u0 = E.pload(m, st.id)
    b0 = E.edge_loads(m, st.id, b0)
    b = gpu_ctx.assemble(u0, b0)
    x, _ = gpu_ctx.solve(b, tol=1e-11)
    u = gpu_ctx.update(x, u0)
    t_host = gpu_ctx.stress(u)
    gpu_ctx.set_state(None, None)
    gpu_ctx.set_loads(m.f, m.eload, m.loadvec)
    gpu_ctx.assemble_resident()
    gpu_ctx.solve_resident(tol=1e-11)
    gpu_ctx.update_resident()
    u_dev, _ = gpu_ctx.state()
    assert np.array_equal(u_dev, u)
    assert np.array_equal(gpu_ctx.stress(None), t_host)
