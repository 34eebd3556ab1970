"""The C ABI library loads and exports every function include/*.h declares.
No compute call: this runs without a GPU."""
import glob
import os
import re

import pytest

import elastic_gb300 as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(elx_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("elx_create", "elx_set_mesh", "elx_set_structure", "elx_assemble",
                     "elx_solve", "elx_destroy", "elx_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, missing


def test_version_string(built_lib):
    assert b"sm_103a" in E.load().elx_version()


def test_no_silent_fallback_without_a_gpu(built_lib):
    """Without a CUDA device the library refuses to create a context."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(E.ElasticError):
        E.Context()
