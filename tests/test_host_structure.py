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


def test_full_size_cube_structure_properties():
    """64^3 HEXA8 (811,200 equations): the structure at full size, checked by
    size-independent properties (sizes, sorted strictly-lower rows, RCM a
    permutation) -- the oracle's O(row^2) sort would take minutes here."""
    m = M.cube_hexa8_64()
    sp = E.host_structure(m, True)
    assert (sp.neq, sp.nad) == (811200, 31442295)
    assert np.array_equal(np.sort(sp.perm), np.arange(1, m.nnode + 1))
    rows = np.repeat(np.arange(1, sp.neq + 1), np.diff(sp.ia))
    assert np.all(sp.ja < rows)
    same_row = rows[1:] == rows[:-1]
    assert np.all(sp.ja[1:][same_row] > sp.ja[:-1][same_row])
