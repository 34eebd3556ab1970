"""Generates tests/golden/pins.json: known answers for the element stiffness
matrices and the RCM ordering that do not come from the oracle.

  python tests/golden/make_pins.py

Element matrices (mef/src/Elmlib02.f: elmt02/03 TRIA3, elmt04/05 QUAD4,
elmt06 TETRA4, elmt07 HEXA8; isw = 2), in exact rational arithmetic:
  * TRIA3 and TETRA4: the constant-strain closed form K = A B^T D B (area or
    volume A, B the constant strain-displacement matrix of the linear shape
    functions) -- the reference's TRIA3 leaves the thickness out of K
    (Elmlib02.f:463-492), its TETRA4 takes the volume as det / 6;
  * QUAD4 on a rectangle and HEXA8 on a box: K = integral of B^T D B over
    the element, integrated exactly (the bilinear / trilinear fields make
    the integrand a polynomial; the reference's 2x2 / 2x2x2 Gauss rule is
    exact for it); QUAD4 plane stress times the thickness (Elmlib02.f:1071).
  D: plane strain E / ((1 + nu)(1 - 2 nu)) [[1 - nu, nu, 0], [nu, 1 - nu, 0],
  [0, 0, (1 - 2 nu) / 2]]; plane stress E / (1 - nu^2) [[1, nu, 0],
  [nu, 1, 0], [0, 0, (1 - nu) / 2]]; 3-D isotropic with lambda, mu.
  Node orders are the reference's (QUAD4 counter-clockwise from (+,+);
  HEXA8 (+,+,+), (-,+,+), (-,-,+), (+,-,+), then the t = -1 face; TETRA4
  with det(x1 - x4, x2 - x4, x3 - x4) > 0), dofs node-major.

RCM (Reord.f:1-435, genrcm / fnroot / rootls / rcm of George and Liu's
SPARSPAK): orderings of small graphs worked out by hand from those rules
(level structures, the minimum-degree node of the last level, neighbours
taken in increasing degree with a stable insertion sort, the component's
Cuthill-McKee order reversed), written below with each derivation.  A
graph is given as TRIA3 connectivity; an element (a, b, b) contributes the
single edge a-b.
"""
from __future__ import annotations

import json
import os

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))


def d_plane(E, nu, stress):
    if stress:
        c = E / (1 - nu ** 2)
        return c * sp.Matrix([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
    c = E / ((1 + nu) * (1 - 2 * nu))
    return c * sp.Matrix([[1 - nu, nu, 0], [nu, 1 - nu, 0], [0, 0, (1 - 2 * nu) / 2]])


def d_solid(E, nu):
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    D = sp.zeros(6, 6)
    for i in range(3):
        for j in range(3):
            D[i, j] = lam + (2 * mu if i == j else 0)
        D[3 + i, 3 + i] = mu
    return D


def b_plane(grads):
    """3 x 2n strain-displacement matrix from the shape-function gradients."""
    n = len(grads)
    B = sp.zeros(3, 2 * n)
    for a, (gx, gy) in enumerate(grads):
        B[0, 2 * a], B[1, 2 * a + 1] = gx, gy
        B[2, 2 * a], B[2, 2 * a + 1] = gy, gx
    return B


def b_solid(grads):
    n = len(grads)
    B = sp.zeros(6, 3 * n)
    for a, (gx, gy, gz) in enumerate(grads):
        B[0, 3 * a], B[1, 3 * a + 1], B[2, 3 * a + 2] = gx, gy, gz
        B[3, 3 * a], B[3, 3 * a + 1] = gy, gx
        B[4, 3 * a + 1], B[4, 3 * a + 2] = gz, gy
        B[5, 3 * a], B[5, 3 * a + 2] = gz, gx
    return B


def linear_gradients(pts):
    """Gradients of the linear shape functions of a simplex (rows: nodes)."""
    n = len(pts)
    M = sp.Matrix([[1] + list(p) for p in pts])
    inv = M.inv()  # N_a = sum_k inv[k, a] * (1, x, y[, z])_k
    return [tuple(inv[k, a] for k in range(1, n)) for a in range(n)], M.det()


def tria3(pts, E, nu, stress):
    g, det = linear_gradients(pts)
    B = b_plane(g)
    return (det / 2) * B.T * d_plane(E, nu, stress) * B


def tetra4(pts, E, nu):
    g, _ = linear_gradients(pts)
    x = [sp.Matrix(p) for p in pts]
    vol = sp.Matrix.hstack(x[0] - x[3], x[1] - x[3], x[2] - x[3]).det() / 6
    B = b_solid(g)
    return vol * B.T * d_solid(E, nu) * B


def quad4_rect(a, b, E, nu, stress, thick):
    """Rectangle [0, a] x [0, b], nodes (a, b), (0, b), (0, 0), (a, 0)."""
    x, y = sp.symbols("x y")
    corners = [(a, b), (0, b), (0, 0), (a, 0)]
    N = [(x / a if cx else 1 - x / a) * (y / b if cy else 1 - y / b) for cx, cy in corners]
    B = b_plane([(sp.diff(n, x), sp.diff(n, y)) for n in N])
    K = (B.T * d_plane(E, nu, stress) * B).applyfunc(
        lambda e: sp.integrate(sp.integrate(sp.expand(e), (x, 0, a)), (y, 0, b)))
    return K * (thick if stress else 1)


def hexa8_box(a, b, c, E, nu):
    """Box [0, a] x [0, b] x [0, c] in the reference's node order."""
    x, y, z = sp.symbols("x y z")
    corners = [(1, 1, 1), (0, 1, 1), (0, 0, 1), (1, 0, 1),
               (1, 1, 0), (0, 1, 0), (0, 0, 0), (1, 0, 0)]
    f = lambda s, c1, L: s / L if c1 else 1 - s / L
    N = [f(x, cx, a) * f(y, cy, b) * f(z, cz, c) for cx, cy, cz in corners]
    B = b_solid([(sp.diff(n, x), sp.diff(n, y), sp.diff(n, z)) for n in N])
    K = (B.T * d_solid(E, nu) * B).applyfunc(
        lambda e: sp.integrate(sp.expand(e), (x, 0, a), (y, 0, b), (z, 0, c)))
    return K


def as_list(K):
    return [[float(v) for v in K.row(i)] for i in range(K.rows)]


def element_pins():
    R = sp.Rational
    E, nu = R(2), R(3, 10)
    tri_unit = [(0, 0), (1, 0), (0, 1)]
    tri_gen = [(R(1, 5), R(-1, 10)), (R(13, 10), R(1, 4)), (R(2, 5), R(11, 10))]
    tet_unit = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 0, 0)]
    tet_gen = [(R(11, 10), R(1, 10), 0), (R(-1, 5), R(9, 10), R(1, 10)),
               (R(1, 10), R(-1, 10), R(6, 5)), (0, 0, 0)]
    out = {}
    for name, pts in (("unit", tri_unit), ("general", tri_gen)):
        for iel, stress in ((2, False), (3, True)):
            out[f"tria3_{name}_iel{iel}"] = {
                "iel": iel, "E": float(E), "nu": float(nu), "thick": 2.0,
                "xl": [[float(v) for v in p] for p in pts],
                "K": as_list(tria3(pts, E, nu, stress))}
    for iel, stress in ((4, False), (5, True)):
        a, b, t = R(2), R(1), R(3, 2)
        out[f"quad4_rect_iel{iel}"] = {
            "iel": iel, "E": float(E), "nu": float(nu), "thick": float(t),
            "xl": [[float(a), float(b)], [0.0, float(b)], [0.0, 0.0], [float(a), 0.0]],
            "K": as_list(quad4_rect(a, b, E, nu, stress, t))}
    for name, pts in (("unit", tet_unit), ("general", tet_gen)):
        out[f"tetra4_{name}"] = {"iel": 6, "E": float(E), "nu": float(nu), "thick": 1.0,
                                 "xl": [[float(v) for v in p] for p in pts],
                                 "K": as_list(tetra4(pts, E, nu))}
    a, b, c = R(1), R(2), R(3, 2)
    corners = [(1, 1, 1), (0, 1, 1), (0, 0, 1), (1, 0, 1),
               (1, 1, 0), (0, 1, 0), (0, 0, 0), (1, 0, 0)]
    out["hexa8_box"] = {"iel": 7, "E": float(E), "nu": float(nu), "thick": 1.0,
                        "xl": [[float(cx * a), float(cy * b), float(cz * c)]
                               for cx, cy, cz in corners],
                        "K": as_list(hexa8_box(a, b, c, E, nu))}
    return out


# Each case: nnode, TRIA3 connectivity (1-based), expected perm (perm[k] =
# the old node at new position k, 1-based), and how it follows from the rules.
RCM_CASES = {
    "path_3_1_4_2": {
        "nnode": 4, "elements": [[3, 1, 1], [1, 4, 4], [4, 2, 2]],
        "perm": [3, 1, 4, 2],
        "derivation": "root 1: levels {1},{3,4},{2} (3 < 4 nodes); last level's min-degree "
                      "node 2 gives 4 levels: root 2; CM from 2: 2,4,1,3; reversed"},
    "star_1": {
        "nnode": 5, "elements": [[1, 2, 2], [1, 3, 3], [1, 4, 4], [1, 5, 5]],
        "perm": [5, 4, 2, 1, 3],
        "derivation": "root 1: 2 levels; first min-degree leaf 2: 3 levels; from there leaf 3 "
                      "(first of {3,4,5}): 3 levels, no gain: root 3; CM 3,1,2,4,5; reversed"},
    "two_components": {
        "nnode": 5, "elements": [[1, 3, 3], [2, 5, 5], [5, 4, 4]],
        "perm": [3, 1, 4, 5, 2],
        "derivation": "component {1,3}: a path from 1 (levels = size): CM 1,3 -> 3,1; "
                      "component {2,5,4}: path from 2: CM 2,5,4 -> 4,5,2"},
    "degree_sort": {
        "nnode": 5, "elements": [[1, 2, 2], [2, 3, 4], [3, 5, 5]],
        "perm": [1, 2, 4, 3, 5],
        "derivation": "root 1: levels {1},{2},{3,4},{5}; last level's node 5: 4 levels, no "
                      "gain: root 5; CM from 5: 3, then 3's neighbours 2 (degree 3) and 4 "
                      "(degree 2) sorted by degree: 4, 2; then 1: 5,3,4,2,1; reversed"},
    "two_quads": {
        "nnode": 6, "quad4": True, "elements": [[1, 2, 5, 4], [2, 3, 6, 5]],
        "perm": [4, 1, 5, 2, 6, 3],
        "derivation": "root 1: levels {1},{2,4,5},{3,6}; min degree of {3,6} (3 and 3): node "
                      "3; its levels {3},{2,5,6},{1,4}: no gain: root 3; CM: 3's neighbours "
                      "2 (5), 5 (5), 6 (3) sorted: 6, 2, 5; then 2's 1, 4: 3,6,2,5,1,4; "
                      "reversed"},
}


def main():
    pins = {"elements": element_pins(), "rcm": RCM_CASES}
    with open(os.path.join(HERE, "pins.json"), "w") as fh:
        json.dump(pins, fh, indent=1)
    print("wrote", os.path.join(HERE, "pins.json"))


if __name__ == "__main__":
    main()
