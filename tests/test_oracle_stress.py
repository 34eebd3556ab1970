"""The oracle's stress recovery (tform_mec, Pform.f:258-421, with the
elements' isw = 3) against exact answers: a linear displacement field gives
every element the same constant strain, so every node's averaged stress is
D eps exactly (patch test, distorted meshes); a rigid rotation gives zero
stress."""
import numpy as np
import pytest

import oracle as O
from elastic_gb300 import meshgen as M

MESHES = {
    "tria3_strain": lambda: M.box2d(7, 5, 2.0, 1.0, etype=M.TRIA3_STRAIN, E=3.0, nu=0.25),
    "tria3_stress": lambda: M.box2d(7, 5, 2.0, 1.0, etype=M.TRIA3_STRESS, E=3.0, nu=0.25),
    "quad4_strain": lambda: M.box2d(6, 4, 2.0, 1.0, etype=M.QUAD4_STRAIN, E=2.0, nu=0.3),
    "quad4_stress": lambda: M.box2d(6, 4, 2.0, 1.0, etype=M.QUAD4_STRESS, E=2.0, nu=0.3),
    "tetra4": lambda: M.box_tetra4(4, 3, 3, jitter=0.2, seed=2),
    "hexa8": lambda: M.box_hexa8(4, 3, 3, jitter=0.2, seed=2),
}


def _distort2d(m, seed):
    rng = np.random.default_rng(seed)
    x = m.x.copy()
    inner = (x[:, 0] > 0) & (x[:, 0] < x[:, 0].max()) & (x[:, 1] > 0) & (x[:, 1] < x[:, 1].max())
    x[inner] += rng.uniform(-0.06, 0.06, size=(int(inner.sum()), 2))
    m.x = x
    return m


def _expected(m, A):
    E, nu = m.e[0, 0], m.e[0, 1]
    iel = int(m.ie[0])
    if m.ndm == 3:
        a1, a2, a3 = 1 - nu, 1 - 2 * nu, 1 + nu
        a, b, c = E * a1 / (a3 * a2), nu / a1, 0.5 * a2 / a1
        e = [A[0, 0], A[1, 1], A[2, 2], A[0, 1] + A[1, 0], A[1, 2] + A[2, 1], A[0, 2] + A[2, 0]]
        return np.array([(e[0] + b * e[1] + b * e[2]) * a, (b * e[0] + e[1] + b * e[2]) * a,
                         (b * e[0] + b * e[1] + e[2]) * a, e[3] * c * a, e[4] * c * a,
                         e[5] * c * a])
    if iel in (M.TRIA3_STRESS, M.QUAD4_STRESS):
        a, b, c = E / (1 - nu * nu), nu, 0.5 * (1 - nu)
    else:
        a1, a2, a3 = 1 - nu, 1 - 2 * nu, 1 + nu
        a, b, c = E * a1 / (a3 * a2), nu / a1, 0.5 * a2 / a1
    e = [A[0, 0], A[1, 1], A[0, 1] + A[1, 0]]
    s1, s2 = a * e[0] + a * b * e[1], a * b * e[0] + a * e[1]
    s3 = nu * (s1 + s2) if iel in (M.TRIA3_STRAIN, M.QUAD4_STRAIN) else 0.0
    return np.array([s1, s2, s3, a * c * e[2]])


@pytest.mark.parametrize("name", sorted(MESHES))
def test_linear_field_gives_exact_stress(name):
    m = MESHES[name]()
    if m.ndm == 2:
        m = _distort2d(m, 3)
    A = np.random.default_rng(4).uniform(-1e-3, 1e-3, (m.ndm, m.ndm))
    u = m.x @ A.T + 0.01
    t = O.tform(m, u)
    expect = _expected(m, A)
    assert np.abs(t - expect).max() <= 1e-10 * np.abs(expect).max()


@pytest.mark.parametrize("name", sorted(MESHES))
def test_rigid_rotation_is_stress_free_and_tx0_added(name):
    m = MESHES[name]()
    W = np.random.default_rng(5).uniform(-1e-3, 1e-3, (m.ndm, m.ndm))
    W = W - W.T  # infinitesimal rotation
    u = m.x @ W.T
    ntn = 4 if m.ndm == 2 else 6
    tx0 = np.random.default_rng(6).standard_normal((m.nnode, ntn))
    t = O.tform(m, u, tx0)
    assert np.abs(t - tx0).max() <= 1e-12
