"""The oracle's restatement of the result writer (write_mesh_res_mec,
Write_vtk.f:742-985 with Vtk.f): the Fortran edit descriptors it prints
(known answers from the Ew.d / Ew.dEe rules: 0.ddddd mantissa, exponent
forms, ties to even, asterisks), and the two files it writes read back
(the XML VTU ASCII file as XML, the legacy binary file record by record)."""
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import oracle as O
from elastic_gb300 import meshgen as M

KNOWN = [
    # value, w, d, e, field
    (1.5, 15, 5, 0, "    0.15000E+01"),
    (-1.5, 15, 5, 0, "   -0.15000E+01"),
    (0.0, 15, 5, 0, "    0.00000E+00"),
    (-0.0, 15, 5, 0, "   -0.00000E+00"),
    (0.0, 15, 5, 3, "   0.00000E+000"),
    (1e-120, 15, 5, 0, "    0.10000-119"),   # Ew.d: 99 < |exp| <= 999 drops the E
    (1e100, 15, 5, 3, "   0.10000E+101"),
    (0.0390625, 15, 5, 0, "    0.39062E-01"),  # exact tie, to even
    (99999950000.0, 15, 5, 3, "   0.10000E+012"),  # exact tie, to even: carries
    (123456.5, 15, 5, 0, "    0.12346E+06"),
    (-2.5e-05, 15, 5, 3, "  -0.25000E-004"),
    (5e-324, 15, 5, 3, "   0.49407E-323"),
    (1.7976931348623157e308, 15, 5, 0, "    0.17977+309"),
    (float("nan"), 15, 5, 0, "            NaN"),
    (float("-inf"), 15, 5, 3, "      -Infinity"),
    (1e-120, 15, 5, 1, "***************"),  # exponent does not fit E1
    (-0.5, 11, 5, 0, "-.50000E+00"),        # no room for the optional zero
]


@pytest.mark.parametrize("v,w,d,e,field", KNOWN)
def test_fortran_edit_descriptors(v, w, d, e, field):
    assert O.fortran_e([v], w, d, e)[0] == field


def _solved(m):
    rng = np.random.default_rng(2)
    u = rng.standard_normal((m.nnode, m.ndf)) * 1e-3
    return u, O.tform(m, u)


MESHES = {
    "quad4": lambda: M.box2d(5, 3, 2.0, 1.0, etype=M.QUAD4_STRESS),
    "tria3": lambda: M.box2d(4, 3, 1.0, 1.0, etype=M.TRIA3_STRAIN),
    "tetra4": lambda: M.box_tetra4(3, 2, 2, jitter=0.1, seed=1),
    "hexa8": lambda: M.box_hexa8(3, 3, 2, jitter=0.1, seed=2),
}
NNOEL = {"quad4": (4, 9), "tria3": (3, 5), "tetra4": (4, 10), "hexa8": (8, 12)}


@pytest.mark.parametrize("name", sorted(MESHES))
def test_vtu_ascii_reads_back(tmp_path, name):
    m = MESHES[name]()
    u, t = _solved(m)
    p = tmp_path / "r.vtu"
    O.write_mesh_res(str(p), m, u, t, fmt=0)
    root = ET.parse(p).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == m.nnode
    assert int(piece.get("NumberOfCells")) == m.numel
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=float)
              for a in root.iter("DataArray") if a.get("Name")}
    pts = np.array(piece.find("Points/DataArray").text.split(), float).reshape(-1, 3)
    assert np.allclose(pts[:, :m.ndm], m.x, rtol=5e-5, atol=1e-300)
    nn, ct = NNOEL[name]
    conn = arrays["connectivity"].reshape(m.numel, nn).astype(int)
    assert np.array_equal(conn, m.ix[:, :nn] - 1)
    assert np.array_equal(arrays["offsets"], nn * np.arange(1, m.numel + 1))
    assert set(arrays["types"]) == {ct}
    assert np.array_equal(arrays["mat"], m.ix[:, m.nen])
    assert np.array_equal(arrays["noIdG"], np.arange(1, m.nnode + 1))
    assert np.allclose(arrays["desloc"].reshape(m.nnode, m.ndf), u, rtol=5e-5)
    st = arrays["stress"].reshape(m.nnode, 9)
    xy = t[:, 3]
    assert np.allclose(st[:, 0], t[:, 0], rtol=5e-5) and np.allclose(st[:, 1], xy, rtol=5e-5)
    assert np.allclose(st[:, 3], xy, rtol=5e-5) and np.allclose(st[:, 8], t[:, 2], rtol=5e-5)


@pytest.mark.parametrize("name", sorted(MESHES))
def test_legacy_binary_reads_back(tmp_path, name):
    m = MESHES[name]()
    u, t = _solved(m)
    p = tmp_path / "r.vtk"
    O.write_mesh_res(str(p), m, u, t, fmt=1)
    raw = p.read_bytes()
    head = b"# vtk DataFile Version 3.0\n" + b"Malha Res".ljust(30) + b"\nBINARY\n"
    assert raw.startswith(head + b"DATASET UNSTRUCTURED_GRID\n")
    pos = raw.index(b" double\n") + 8
    pts = np.array(struct.unpack(">%dd" % (3 * m.nnode), raw[pos:pos + 24 * m.nnode]))
    assert np.array_equal(pts.reshape(-1, 3)[:, :m.ndm], m.x)
    nn, ct = NNOEL[name]
    pos = raw.index(b"\nCELLS ") + 7 + 30 + 1
    cells = np.array(struct.unpack(">%di" % ((nn + 1) * m.numel),
                                   raw[pos:pos + 4 * (nn + 1) * m.numel])).reshape(m.numel, -1)
    assert np.all(cells[:, 0] == nn) and np.array_equal(cells[:, 1:], m.ix[:, :nn] - 1)
    pos = raw.index(b" TENSORS stress          double\n") + 32
    st = np.array(struct.unpack(">%dd" % (9 * m.nnode), raw[pos:pos + 72 * m.nnode]))
    assert np.array_equal(st.reshape(-1, 9)[:, 0], t[:, 0])
    assert len(raw) == pos + 72 * m.nnode


def test_mixed_cell_types_refused(tmp_path):
    m = MESHES["quad4"]()
    m.ie = np.array([M.QUAD4_STRESS, M.TRIA3_STRESS], np.int32)
    m.e = np.repeat(m.e, 2, axis=0) if m.e.shape[0] == 1 else m.e
    m.ix[0, m.nen] = 2
    with pytest.raises(O.OracleError):
        O.write_mesh_res(str(tmp_path / "x.vtu"), m)
