"""Result writer on the GPU (elx_write_vtk / elx_format_vtk =
write_mesh_res_mec, Write_vtk.f:742-985) against the oracle's restatement:
the device's Ew.d / Ew.dEe fields equal the oracle's (glibc's exact
conversion) for doubles across the whole range, exact decimal ties,
boundaries of powers of ten, subnormals, zeros and non-finite values; the
files (XML VTU ASCII and legacy binary) are byte-identical to the oracle's
for every element type, written from the device's own solve and stresses."""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def _values():
    rng = np.random.default_rng(17)
    v = [0.0, -0.0, np.nan, np.inf, -np.inf, 5e-324, -5e-324, 2.2250738585072014e-308,
         1.7976931348623157e308, 1.0, 0.1, 0.5, 1.5, 2.5, 0.0390625, 99999950000.0,
         0.999995, 0.9999949999999999, 9.99995, 1e-120, 1e100, 1e-100, 1e99, 1e-99]
    v += list(10.0 ** np.arange(-320, 309))            # powers of ten (rounded)
    v += list(np.nextafter(10.0 ** np.arange(-300, 300), np.inf))
    v += list(np.nextafter(10.0 ** np.arange(-300, 300), -np.inf))
    # exact decimal ties at the 6th digit: k/2^j with short expansions
    v += [k / 2.0 ** j for k in range(1, 400, 7) for j in range(1, 24)]
    mags = rng.uniform(-320, 308, 20000)
    v += list(np.sign(rng.standard_normal(mags.size)) * 10.0 ** mags)
    v += list(rng.standard_normal(5000))
    return np.array(v, dtype=np.float64)


@pytest.mark.parametrize("w,d,e", [(15, 5, 0), (15, 5, 3), (12, 5, 0), (22, 9, 4)])
def test_fortran_fields_match_oracle(built_lib, w, d, e):
    x = _values()
    dev = E.fortran_e(x, w, d, e)
    ref = O.fortran_e(x, w, d, e)
    bad = [(float(x[i]), dev[i], ref[i]) for i in range(len(x)) if dev[i] != ref[i]]
    assert not bad, bad[:10]


MESHES = {
    "quad4_stress": lambda: M.cantilever_quad4_64x16(),
    "tria3_strain": lambda: M.box2d(9, 7, 2.0, 1.0, etype=M.TRIA3_STRAIN, E=3.0, nu=0.25),
    "tetra4": lambda: M.box_tetra4(6, 5, 4, jitter=0.2, lognormal_E=True, seed=4),
    "hexa8": lambda: M.box_hexa8(8, 7, 6, jitter=0.2, seed=5),
}


@pytest.mark.parametrize("fmt", [E.VTK_VTU_ASCII, E.VTK_LEGACY_BINARY])
@pytest.mark.parametrize("name", sorted(MESHES))
def test_files_match_oracle_bytewise(gpu_ctx, tmp_path, name, fmt):
    m = MESHES[name]()
    u, _, ctx = E.solvm(m, tol=1e-11, ctx=gpu_ctx)
    t = ctx.stress(u)
    dev = tmp_path / "dev.out"
    n = ctx.write_vtk(str(dev), fmt, E.VTK_DESLOC | E.VTK_STRESS)
    ref = tmp_path / "ref.out"
    O.write_mesh_res(str(ref), m, u, t, fmt)
    assert n == ref.stat().st_size
    assert dev.read_bytes() == ref.read_bytes()
    # fields switched off, and the in-memory form
    for fields, uu, tt in [(0, None, None), (E.VTK_DESLOC, u, None), (E.VTK_STRESS, None, t)]:
        O.write_mesh_res(str(ref), m, uu, tt, fmt)
        assert ctx.format_vtk(fmt, fields) == ref.read_bytes()


def test_writer_errors(built_lib, tmp_path):
    ctx = E.Context(device=0)
    try:
        m = MESHES["hexa8"]()
        ctx.set_mesh(m)
        ctx.build_structure(True)
        with pytest.raises(E.ElasticError) as e:  # no stresses computed yet
            ctx.format_vtk(E.VTK_VTU_ASCII, E.VTK_STRESS)
        assert e.value.code == E.ERR_STATE
        with pytest.raises(E.ElasticError) as e:
            ctx.format_vtk(2, 0)
        assert e.value.code == E.ERR_ARG
        with pytest.raises(E.ElasticError) as e:
            ctx.write_vtk(str(tmp_path / "missing" / "dir" / "x.vtu"), E.VTK_VTU_ASCII, 0)
        assert e.value.code == E.ERR_ARG
    finally:
        ctx.close()
