"""Generates the golden fixtures in this directory from the reference's own
example decks (lmn-labest/Elastic, input/) and the CPU oracle.

Run with the reference project's checkout as the argument (or in the
ELASTIC_REFERENCE environment variable):
    python tests/golden/make_golden.py <path to lmn-labest/Elastic>

It writes
  decks.npz     the 3-D HEXA8 / TETRA4 deck meshes (caso_a, nodal forces), in
                the layout of elastic_gb300.meshgen.Mesh, so that GPU tests can
                use the reference's own meshes on a machine without the decks;
  golden.json   per deck: sizes, structure checksums, oracle PCG results.

Deck format (mef/src/Rdata.f): macro words, `insert <file>` relative to the
deck (Rdata.f:561-568), `return` ends an inserted file, `//` comments.
The decks' inline `config ... end config` block and the `pcg ...` line are
skipped (the reference itself cannot read the former, see Rdata.f:1918).
"""
from __future__ import annotations

import hashlib
import re
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from elastic_gb300 import meshgen as M  # noqa: E402
import oracle as O  # noqa: E402

ELEM_NODES = {"tria3": 3, "quad4": 4, "tetra4": 4, "hexa8": 8}


def _lines(path):
    base = os.path.dirname(path)
    with open(path) as f:
        for raw in f:
            line = raw.strip()
            if not line or line.startswith("//"):
                continue
            w = line.split()
            if w[0] == "insert":
                yield from _lines(os.path.join(base, w[1]))
                continue
            if w[0] == "return":
                return
            yield w


def _num(s):
    # Fortran reals: 1.0d0, 0.3369d+00 and the letterless exponent 0.0+00
    s = s.replace("d", "e").replace("D", "e")
    s = re.sub(r"(?<=[0-9.])([+-])(?=[0-9]+$)", r"e\1", s)
    return float(s)


def read_deck(path):
    it = _lines(path)
    hdr = {}
    x = ix = ie = e = idm = f = nload = eload = None
    loads = {}
    etype_name = None
    for w in it:
        k = w[0]
        if k == "config":
            for w2 in it:
                if w2[0] == "end":
                    break
        elif k == "mesh":
            w2 = next(it)
            hdr = {w2[i]: int(w2[i + 1]) for i in range(0, len(w2) - 1, 2)}
            nnode, numel, numat = hdr["nnode"], hdr["numel"], hdr["numat"]
            ndf, ndm, nen = hdr["ndf"], hdr["dim"], hdr["maxno"]
            x = np.zeros((nnode, ndm))
            ix = np.zeros((numel, nen + 1), np.int32)
            ie = np.zeros(numat, np.int32)
            e = np.zeros((numat, M.PROP))
            idm = np.zeros((nnode, ndf), np.int32)
            f = np.zeros((nnode, ndf))
            nload = np.zeros((nnode, ndf), np.int32)
            eload = np.zeros((numel, 7), np.int32)
        elif k == "materials":
            for w2 in it:
                if w2[0] == "end":
                    break
                ma = int(w2[0])
                ie[ma - 1] = int(w2[1])
                vals = [_num(v) for v in w2[2:]]
                e[ma - 1, :len(vals)] = vals
        elif k == "coordinates":
            for w2 in it:
                if w2[0] == "end":
                    break
                n = int(w2[0])
                x[n - 1] = [_num(v) for v in w2[1:1 + x.shape[1]]]
        elif k in ELEM_NODES:
            etype_name = k
            nv = ELEM_NODES[k]
            for w2 in it:
                if w2[0] == "end":
                    break
                el = int(w2[0])
                ix[el - 1, :nv] = [int(v) for v in w2[1:1 + nv]]
                ix[el - 1, -1] = int(w2[1 + nv])
        elif k == "constraindisp":
            for w2 in it:
                if w2[0] == "end":
                    break
                n = int(w2[0])
                v = [int(t) for t in w2[1:]]
                idm[n - 1, :len(v)] = v
        elif k == "nodalforces":
            for w2 in it:
                if w2[0] == "end":
                    break
                n = int(w2[0])
                v = [_num(t) for t in w2[1:]]
                f[n - 1, :len(v)] = v
        elif k == "nodalloads":
            for w2 in it:
                if w2[0] == "end":
                    break
                n = int(w2[0])
                v = [int(t) for t in w2[1:]]
                nload[n - 1, :len(v)] = v
        elif k == "elmtloads":
            for w2 in it:
                if w2[0] == "end":
                    break
                el = int(w2[0])
                v = [int(t) for t in w2[1:]]
                eload[el - 1, :len(v)] = v
        elif k == "loads":
            for w2 in it:
                if w2[0] == "end":
                    break
                lid, ltype = int(w2[0]), int(w2[1])
                if ltype == 1:
                    loads[lid] = ("const", _num(w2[2]))
                elif ltype == 40:
                    npar = int(w2[2])
                    loads[lid] = ("vec", [_num(t) for t in w2[3:3 + npar]])
                else:
                    raise ValueError(f"load type {ltype} not handled")
        elif k == "end" and len(w) > 1 and w[1] == "mesh":
            break
    # nodal loads (tload type 1, Pload.f:136-138): f(j,i) = c
    for (n, j) in zip(*np.nonzero(nload)):
        kind, val = loads[int(nload[n, j])]
        f[n, j] = val
    loadvec = None
    if eload.any():
        nl = max(loads) if loads else 0
        loadvec = np.zeros((nl, 2))
        for lid, (kind, val) in loads.items():
            if kind == "vec":
                loadvec[lid - 1, :len(val)] = val[:2]
    else:
        eload = None
    return M.Mesh(ndm=x.shape[1], ndf=idm.shape[1], nen=ix.shape[1] - 1, x=x, ix=ix, ie=ie,
                  e=e, id=idm, f=f, eload=eload, loadvec=loadvec,
                  name=os.path.basename(path))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def main(ref):
    inp = os.path.join(ref, "input")
    decks = {
        "quad_el": "quad/exemplo1_apostila_el.dat",
        "quad_el_ept": "quad/exemplo1_apostila_el_ept.dat",
        "quad_nf": "quad/exemplo1_apostila_nf.dat",
        "quad_nl": "quad/exemplo1_apostila_nl.dat",
        "hexa_nf": "hexa/linear/caso_a/solo1_mec_nf.dat",
        "hexa_nl": "hexa/linear/caso_a/solo1_mec_nl.dat",
        "tetra_nf": "tetra/linear/caso_a/solo1_tetra_mec_nf.dat",
        "tetra_nl": "tetra/linear/caso_a/solo1_tetra_mec_nl.dat",
    }
    out = {"source": "reference input decks + oracle (oracle/elx_oracle.c)",
           "tol": 1e-11, "decks": {}}
    arrays = {}
    for key, rel in decks.items():
        m = read_deck(os.path.join(inp, rel))
        u, info, s, ad, al = O.solvm(m, tol=1e-11)
        rec = {
            "deck": rel, "nnode": m.nnode, "numel": m.numel, "neq": s.neq, "nad": s.nad,
            "perm_sha": sha(s.perm), "id_sha": sha(s.id), "ia_sha": sha(s.ia), "ja_sha": sha(s.ja),
            "iters": info["iters"], "xkx": info["xkx"], "sqrt_xkx": float(np.sqrt(info["xkx"])),
            "norm_x": info["norm_x"], "norm_r": info["norm_r"], "norm_m_r": info["norm_m_r"],
            "u_max_abs": float(np.abs(u).max()), "u_sum": float(u.sum()),
            "ad_sum": float(ad.sum()), "al_sum": float(al.sum()),
        }
        if key.startswith("quad"):
            g = M.square_quad4_100(plane_stress=(key == "quad_el_ept"))
            same = (np.array_equal(g.ix, m.ix) and np.allclose(g.x, m.x, atol=0, rtol=0)
                    and np.array_equal(g.id, m.id) and np.array_equal(g.ie, m.ie)
                    and np.allclose(g.e[:, :2], m.e[:, :2]))
            rec["generator_matches_deck_geometry"] = bool(same)
        if key in ("hexa_nf", "tetra_nf", "hexa_nl", "tetra_nl"):
            for name in ("x", "ix", "ie", "e", "id", "f"):
                arrays[f"{key}__{name}"] = getattr(m, name)
        out["decks"][key] = rec
        print(key, rec["neq"], rec["nad"], rec["iters"], rec["sqrt_xkx"])
    np.savez_compressed(os.path.join(HERE, "decks.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


def load_deck_mesh(key):
    """Mesh of a 3-D deck stored in decks.npz (no reference needed)."""
    z = np.load(os.path.join(HERE, "decks.npz"))
    ix = z[f"{key}__ix"]
    return M.Mesh(ndm=3, ndf=3, nen=ix.shape[1] - 1, x=z[f"{key}__x"], ix=ix,
                  ie=z[f"{key}__ie"], e=z[f"{key}__e"], id=z[f"{key}__id"], f=z[f"{key}__f"],
                  name=key)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ELASTIC_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set ELASTIC_REFERENCE)")
    main(ref)
