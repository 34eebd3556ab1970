"""The partitioned product on one GPU (elx_partition_spmv): every partition
gathers its halo and multiplies its owned block rows on its local numbering
(matvec_csrcrsym1, Matvec.f:1090-1191); the assembled y is bitwise the
single-partition FP64 product, each partition's rows are within 1e-14 of
the oracle's matvec_csrcrsym1 on that partition's host arrays (the lower
CSRC and the rectangular part on its local numbering, with the halo of x),
and the device partitions are the host partitions (elx_host_partition_*:
same cuts, same halo)."""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rel_inf, rollers

pytestmark = pytest.mark.gpu

MESHES = {
    "hexa8": lambda: M.box_hexa8(11, 9, 8, jitter=0.2, seed=5),
    "tetra4": lambda: M.box_tetra4(8, 7, 6, jitter=0.2, lognormal_E=True, seed=4),
    "quad4": lambda: M.box2d(60, 40, 2.0, 1.0, etype=M.QUAD4_STRESS),
    "tria3": lambda: M.box2d(50, 30, 2.0, 1.0, etype=M.TRIA3_STRAIN),
}


@pytest.mark.parametrize("nparts", [1, 2, 3, 7])
@pytest.mark.parametrize("name", sorted(MESHES))
def test_partitioned_product_is_bitwise_the_product(gpu_ctx, name, nparts):
    m = MESHES[name]()
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    _, ad, al = gpu_ctx.assemble(None, None, want_matrix=True)
    x = np.random.default_rng(nparts).standard_normal(gpu_ctx.sizes()[0])
    y = gpu_ctx.spmv(x)
    yp = gpu_ctx.partition_spmv(x, nparts)
    assert np.array_equal(yp, y)
    for part in range(nparts):
        hp = E.host_partition(m, nparts, part)
        assert gpu_ctx.partition_info(nparts, part) == (hp.eq0, hp.neq, len(hp.halo))
        xl = np.concatenate([x[hp.eq0:hp.eq0 + hp.neq], x[hp.halo]])
        y_o = O.matvec_csrcrsym1(hp.neq, hp.ia, hp.ja, hp.ia1, hp.ja1,
                                 ad[hp.eq0:hp.eq0 + hp.neq], al[hp.pos], al[hp.pos1], xl)
        assert rel_inf(y_o, yp[hp.eq0:hp.eq0 + hp.neq]) <= 1e-14, part


def test_partition_errors(gpu_ctx):
    m = rollers(M.box_hexa8(4, 4, 4))  # partly fixed nodes: no node blocks
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    gpu_ctx.assemble(None, None)
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.partition_spmv(np.ones(gpu_ctx.sizes()[0]), 2)
    assert e.value.code == E.ERR_ARG
    m = M.box_hexa8(3, 3, 3)  # 64 nodes: two cut units of 32
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    gpu_ctx.assemble(None, None)
    x = np.ones(gpu_ctx.sizes()[0])
    assert np.array_equal(gpu_ctx.partition_spmv(x, 2), gpu_ctx.spmv(x))
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.partition_spmv(x, 3)
    assert e.value.code == E.ERR_ARG
