"""The library's host-side structure code (node graph, RCM, numeq, lower
CSRC pattern) against the oracle: bit for bit.  CPU only (no GPU call)."""
import json
import os
import sys

import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import relabel_nodes, two_components

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _same(m, reorder):
    so = O.structure(m, reorder)
    sp = E.host_structure(m, reorder)
    assert (so.neq, so.nad) == (sp.neq, sp.nad)
    assert np.array_equal(so.perm, sp.perm), "RCM permutation differs"
    assert np.array_equal(so.id, sp.id), "equation numbering differs"
    assert np.array_equal(so.ia, sp.ia), "ia differs"
    assert np.array_equal(so.ja, sp.ja), "ja differs"
    return so


MESHES = {
    "quad4_cantilever": lambda: M.cantilever_quad4_64x16(),
    "quad4_square": lambda: M.square_quad4_100(),
    "tria3": lambda: M.box2d(9, 6, etype=M.TRIA3_STRAIN, clamp="bottom"),
    "tetra4_jitter": lambda: M.box_tetra4(6, 5, 4, jitter=0.2, lognormal_E=True),
    "hexa8": lambda: M.box_hexa8(7, 6, 5),
    "hexa8_scrambled": lambda: relabel_nodes(M.box_hexa8(6, 5, 4), 3),
    "tetra4_scrambled": lambda: relabel_nodes(M.box_tetra4(4, 4, 3), 5),
    "quad4_two_components": lambda: two_components(M.box2d(5, 4)),
    "hexa8_two_components_scrambled": lambda: relabel_nodes(two_components(M.box_hexa8(3, 3, 2)), 9),
}


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("reorder", [True, False])
def test_structure_bit_exact(name, reorder):
    _same(MESHES[name](), reorder)


def test_partially_constrained_nodes():
    m = M.box_hexa8(5, 4, 3)
    rng = np.random.default_rng(2)
    m.id[:] = (rng.uniform(size=m.id.shape) < 0.2).astype(np.int32)
    _same(m, True)


def test_deck_meshes_match_golden_checksums():
    sys.path.insert(0, GOLD)
    from make_golden import load_deck_mesh, sha
    gold = json.load(open(os.path.join(GOLD, "golden.json")))["decks"]
    for key in ("hexa_nf", "tetra_nf"):
        m = load_deck_mesh(key)
        sp = E.host_structure(m, True)
        g = gold[key]
        assert (sp.neq, sp.nad) == (g["neq"], g["nad"])
        assert sha(sp.perm) == g["perm_sha"] and sha(sp.id) == g["id_sha"]
        assert sha(sp.ia) == g["ia_sha"] and sha(sp.ja) == g["ja_sha"]


@pytest.mark.parametrize("name", ["cube_hexa8_64", "cube_tetra4_48_mixed", "plate_hexa8_96"])
def test_full_size_structures_bit_exact(name):
    """The benchmark meshes at full size (811,200 / 345,744 / 1,354,896
    equations): perm, id, ia, ja bit for bit against the oracle."""
    m = getattr(M, name)()
    if isinstance(m, tuple):
        m = m[0]
    _same(m, True)


def test_full_size_cube_structure_properties():
    """64^3 HEXA8 (811,200 equations): sizes, sorted strictly-lower rows,
    RCM a permutation."""
    m = M.cube_hexa8_64()
    sp = E.host_structure(m, True)
    assert (sp.neq, sp.nad) == (811200, 31442295)
    assert np.array_equal(np.sort(sp.perm), np.arange(1, m.nnode + 1))
    rows = np.repeat(np.arange(1, sp.neq + 1), np.diff(sp.ia))
    assert np.all(sp.ja < rows)
    same_row = rows[1:] == rows[:-1]
    assert np.all(sp.ja[1:][same_row] > sp.ja[:-1][same_row])


def colouring_conflicts(mesh, color):
    """Pairs (colour, node) where two elements of one colour share a vertex
    node -- and so an equation, whose entries two threads of one assembly
    launch would then add at once.  The reference's guarantee for its own
    colouring (Colormsh.f:160-247) restated as a check; 0 means race-free."""
    nen1 = mesh.nen + 1
    ix = mesh.ix.reshape(mesh.numel, nen1)
    nv = np.array([M.NEN_OF_TYPE[int(mesh.ie[ix[el, -1] - 1])]
                   for el in range(mesh.numel)])
    seen = {}
    conflicts = 0
    for el in range(mesh.numel):
        for node in ix[el, :nv[el]]:
            key = (int(color[el]), int(node))
            if key in seen:
                conflicts += 1
            seen[key] = el
    return conflicts


COLOUR_MESHES = dict(MESHES, cube_hexa8_24=lambda: M.box_hexa8(24, 24, 24),
                     tetra4_cube=lambda: M.box_tetra4(10, 9, 8, jitter=0.2, seed=3))


@pytest.mark.parametrize("name", sorted(COLOUR_MESHES))
def test_element_colouring_is_race_free(name):
    """No two elements of one colour share a node, every element has a
    colour, and the colours are 1..ncolors."""
    m = COLOUR_MESHES[name]()
    col = E.host_colors(m)
    assert col.min() == 1 and set(np.unique(col)) == set(range(1, col.max() + 1))
    assert colouring_conflicts(m, col) == 0


def test_element_colouring_full_size_cube():
    """The 64^3 HEXA8 cube (262,144 elements): race-free, with the greedy
    colouring's 8 colours of a structured hexahedral mesh, checked with
    array operations (each colour's vertex nodes all distinct)."""
    m = M.cube_hexa8_64()
    col = E.host_colors(m)
    ix = m.ix.reshape(m.numel, m.nen + 1)[:, :8]
    assert col.max() == 8
    for c in range(1, col.max() + 1):
        nodes = ix[col == c].ravel()
        assert np.unique(nodes).size == nodes.size, c


def test_colouring_check_catches_a_shared_node():
    """The check itself: two neighbouring elements put in one colour are
    reported (a mistake planted in a copy of the colours)."""
    m = M.box_hexa8(4, 3, 3)
    col = E.host_colors(m).copy()
    col[1] = col[0]  # elements 0 and 1 share a face
    assert colouring_conflicts(m, col) > 0


def test_threaded_host_structure_is_repeatable():
    """The host structure's per-node and per-element passes run on several
    threads (the graph's neighbour lists are filled in thread order, then
    sorted); a 384,000-element TETRA4 mesh, large enough for them to
    split, gives the same perm, id, ia, ja and colours on every build, and
    the same as the oracle's."""
    m = M.box_tetra4(40, 40, 40, jitter=0.1, seed=11)
    a, b = E.host_structure(m, True), E.host_structure(m, True)
    for k in ("perm", "id", "ia", "ja"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert np.array_equal(E.host_colors(m), E.host_colors(m))
    _same(m, True)
