"""Device memory of the contexts: a stream-ordered pool per device
(cudaMallocFromPoolAsync / cudaFreeAsync on the context's stream) by
default, plain cudaMalloc / cudaFree with ELX_DEVICE_POOL=0 (read once per
device and process, so each variant runs in its own process).

Bar: the two give bitwise the same assembly, PCG, mixed and block solutions
and the same device byte count; contexts created and destroyed in a loop
(the server's pattern) keep giving the same bits.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import elastic_gb300 as E
from elastic_gb300 import meshgen as M
m = M.box_hexa8(10, 9, 8, jitter=0.2, seed=3)
out = {}
for rep in range(3):
    with E.Context(device=0) as ctx:
        ctx.set_mesh(m)
        ctx.build_structure(True)
        neq = ctx.sizes()[0]
        b = ctx.assemble(None, None)
        B = np.random.default_rng(1).standard_normal((neq, 4))
        x, _ = ctx.solve(B[:, 0], tol=1e-10)
        xm, _ = ctx.solve(B[:, 1], precision=E.PREC_MIXED, tol=1e-10)
        X, _ = ctx.solve_block(B, precision=E.PREC_FP64, tol=1e-10, width=4)
        out[rep] = {"x": x.tobytes().hex(), "xm": xm.tobytes().hex(),
                    "X": X.tobytes().hex(), "bytes": ctx.device_bytes}
assert out[0] == out[1] == out[2]
np.savez(sys.argv[2], x=np.frombuffer(bytes.fromhex(out[0]["x"])),
         xm=np.frombuffer(bytes.fromhex(out[0]["xm"])),
         X=np.frombuffer(bytes.fromhex(out[0]["X"])), nbytes=out[0]["bytes"])
"""


def _run(tmp_path, pool):
    env = dict(os.environ, ELX_DEVICE_POOL=pool)
    path = str(tmp_path / f"pool{pool}.npz")
    r = subprocess.run([sys.executable, "-c", SCRIPT, ROOT, path], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


def test_pool_and_plain_allocation_give_the_same_bits(built_lib, tmp_path):
    a, b = _run(tmp_path, "1"), _run(tmp_path, "0")
    for k in ("x", "xm", "X", "nbytes"):
        assert np.array_equal(a[k], b[k]), k
