"""The allocation-free entry point elx_spmv_dot_noalloc, through the C ABI.

It exists for callers that cannot let the library allocate device memory
(a driver that carves every device array out of one pool it allocated up
front, as the reference's memory manager does, or code that must not call
cudaMalloc in the middle of asynchronous work).  Its only scratch is a static
device array shared by all calls.  This file is collected last so that a run
stopping at the first failure has already run every other test; it passes
alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rel_inf

pytestmark = pytest.mark.gpu

SPMV_TOL = 1e-14   # same bar as the SpMV parity tests
DOT_TOL = 1e-13
MAX_ROWS = 1048576


def upper_csr(ia, ja, neq):
    """Transpose of the strict lower part: (iat, jat) 1-based and pt, the
    0-based position in al of each upper entry (counting sort by column)."""
    rows = np.repeat(np.arange(neq), np.diff(ia))
    cols = ja - 1
    order = np.lexsort((rows, cols))          # by column, then row
    counts = np.bincount(cols, minlength=neq)
    iat = np.concatenate([[1], 1 + np.cumsum(counts)]).astype(np.int32)
    return iat, (rows[order] + 1).astype(np.int32), order


def test_noalloc_matches_context_spmv(built_lib):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    m = M.box_hexa8(10, 9, 8, jitter=0.15)
    with E.Context(device=0) as ctx:
        ctx.set_mesh(m)
        neq, nad, _ = ctx.build_structure(True)
        st = ctx.structure()
        _, ad, al = ctx.assemble(None, None, want_matrix=True)
        iat, jat, pt = upper_csr(st.ia, st.ja, neq)
        alt = al[pt]
        to = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
        d = {"ia": to(st.ia, np.int32), "ja": to(st.ja, np.int32), "ad": to(ad, np.float64),
             "al": to(al, np.float64), "iat": to(iat, np.int32), "jat": to(jat, np.int32),
             "alt": to(alt, np.float64)}
        fn = E.load().elx_spmv_dot_noalloc
        ptr = lambda t: C.c_void_p(t.data_ptr())
        rng = np.random.default_rng(11)
        stream = torch.cuda.current_stream(dev)
        for call in range(2):  # two calls in a row share the scratch
            x = rng.standard_normal(neq)
            y_ref = ctx.spmv(x)  # the existing entry point (context, host buffers)
            d_x = to(x, np.float64)
            d_y = torch.full((neq,), np.nan, dtype=torch.float64, device=dev)
            d_xy = torch.full((1,), np.nan, dtype=torch.float64, device=dev)
            rc = fn(neq, ptr(d["ia"]), ptr(d["ja"]), ptr(d["ad"]), ptr(d["al"]), ptr(d["iat"]),
                    ptr(d["jat"]), ptr(d["alt"]), ptr(d_x), ptr(d_y), ptr(d_xy),
                    C.c_void_p(stream.cuda_stream))
            assert rc == E.OK, f"call {call}: status {rc}"
            torch.cuda.synchronize(dev)
            y = d_y.cpu().numpy()
            assert rel_inf(y_ref, y) <= SPMV_TOL, f"call {call}"
            # and the oracle's matvec_csrcsym1 (Matvec.f:528-621) on the same arrays
            s = O.Structure(perm=st.perm, id=st.id, neq=neq, nad=nad, ia=st.ia, ja=st.ja)
            assert rel_inf(O.matvec(s, ad, al, x), y) <= SPMV_TOL, f"call {call}"
            xy_ref = float(x @ y_ref)
            assert abs(d_xy.item() - xy_ref) <= DOT_TOL * abs(xy_ref), f"call {call}"
        # sizes beyond the scratch's maximum are refused before any GPU work
        rc = fn(MAX_ROWS + 1, ptr(d["ia"]), ptr(d["ja"]), ptr(d["ad"]), ptr(d["al"]),
                ptr(d["iat"]), ptr(d["jat"]), ptr(d["alt"]), ptr(d_x), ptr(d_y), ptr(d_xy),
                C.c_void_p(stream.cuda_stream))
        assert rc == E.ERR_ARG
