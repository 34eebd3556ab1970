"""The oracle (and the library's host structure code) against known answers
that do not come from the oracle: tests/golden/pins.json, made by
tests/golden/make_pins.py --

  * element stiffness matrices in exact rational arithmetic: the
    constant-strain closed forms of TRIA3 (plane strain and stress) and
    TETRA4, the exact integral of B^T D B over a rectangular QUAD4 and a box
    HEXA8 (what Elmlib02.f's elmt02-07 compute at isw = 2): within 1e-14 of
    the largest entry (TETRA4 carries the reference's div6 literal,
    0.166666666666667, 2e-15 from 1/6);
  * RCM orderings of small graphs worked out by hand from the rules of
    Reord.f (genrcm, fnroot, rootls, rcm): bit for bit.
"""
import json
import os

import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "pins.json")))


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("name", sorted(PINS["elements"]))
def test_element_stiffness_closed_form(name):
    p = PINS["elements"][name]
    K = np.array(p["K"])
    Ko = O.element_stiffness(p["iel"], [p["E"], p["nu"], p["thick"]], np.array(p["xl"]))
    assert np.abs(Ko - K).max() <= 1e-14 * np.abs(K).max()


def graph_mesh(case):
    """A mesh whose node graph is the case's graph (TRIA3 connectivity; an
    element (a, b, b) contributes the edge a-b; QUAD4 where marked)."""
    els = np.array(case["elements"], dtype=np.int32)
    n = case["nnode"]
    iel = M.QUAD4_STRESS if case.get("quad4") else M.TRIA3_STRESS
    ix = np.hstack([els, np.ones((len(els), 1), np.int32)])
    e = np.zeros((1, M.PROP))
    e[0, :3] = (1.0, 0.3, 1.0)
    return M.Mesh(ndm=2, ndf=2, nen=els.shape[1], x=np.zeros((n, 2)), ix=ix,
                  ie=np.array([iel], np.int32), e=e, id=np.zeros((n, 2), np.int32),
                  f=np.zeros((n, 2)), name="graph")


@pytest.mark.parametrize("name", sorted(PINS["rcm"]))
def test_rcm_hand_derived(name):
    case = PINS["rcm"][name]
    m = graph_mesh(case)
    want = np.array(case["perm"], dtype=np.int32)
    assert np.array_equal(O.structure(m, True).perm, want)
    assert np.array_equal(E.host_structure(m, True).perm, want)
