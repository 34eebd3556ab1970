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


def test_fortran_module_matches_the_header(built_lib):
    """include/elastic_gb300.f90 (the driver's ISO_C_BINDING module) binds
    only exported entry points declared in the header, and its constants
    carry the header's values.  (No Fortran compiler here: a consistency
    check of the text, not a compile.)"""
    f90 = open(os.path.join(ROOT, "include", "elastic_gb300.f90")).read()
    bound = re.findall(r"bind\(C,\s*name='(elx_[a-z0-9_]+)'\)", f90)
    declared = set(declared_functions())
    assert bound and set(bound) <= declared, set(bound) - declared
    assert all(hasattr(built_lib, n) for n in bound)
    for required in ("elx_create", "elx_set_mesh", "elx_set_structure", "elx_assemble",
                     "elx_solve", "elx_destroy", "elx_last_error"):
        assert required in bound
    header = open(os.path.join(ROOT, "include", "elastic_gb300.h")).read()
    defines = dict(re.findall(r"#define (ELX_[A-Z0-9_]+) (-?\d+)", header))
    params = dict(re.findall(r"(ELX_[A-Z0-9_]+) = (-?\d+)", f90))
    for name, value in params.items():
        if name in defines:
            assert defines[name] == value, name
    assert {"ELX_OK", "ELX_SOLVER_PCG", "ELX_SOLVER_BICGSTAB_NOPREC",
            "ELX_PREC_MIXED"} <= set(params)
