"""The C-ABI library: it builds, loads, and exports every entry point that
include/togb.h declares; argument validation needs no GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from tensororder_gb300 import build, runtime


def declared_symbols():
    with open(os.path.join(ROOT, "include", "togb.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(togb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return runtime.lib()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert "togb_program_run" in syms and "togb_tensordot_f64" in syms
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(runtime.EXPORTS)


def header_struct(name):
    """(field, array length or 0) of a typedef struct in include/togb.h."""
    with open(os.path.join(ROOT, "include", "togb.h")) as f:
        text = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    body = re.search(r"typedef struct \{([^}]*)\}\s*" + name + r"\s*;", text).group(1)
    out = []
    for decl in body.split(";"):
        for part in decl.strip().split(","):  # "double w_neg, w_pos" declares two fields
            m = re.search(r"(\w+)\s*(?:\[(\d+)\])?\s*$", part.strip())
            if m:
                out.append((m.group(1), int(m.group(2) or 0)))
    return out


@pytest.mark.parametrize("mirror,name", [(runtime.ProgramInfo, "togb_program_info"),
                                         (runtime.ProgramDesc, "togb_program_desc"),
                                         (runtime.LeafSpec, "togb_leaf_spec")])
def test_ctypes_mirrors_match_the_header(mirror, name):
    fields = [(f, getattr(t, "_length_", 0)) for f, t in mirror._fields_]
    assert fields == header_struct(name)


def test_version(lib):
    assert lib.togb_version() == 1


def _desc(ranks, axes, values, tokens, gsize=(), gedges=()):
    keep = [np.array(x or [0], dtype=np.int32) for x in (ranks, axes, tokens, gsize, gedges)]
    vals = np.array(values or [0.0], dtype=np.float64)
    i32 = ctypes.POINTER(ctypes.c_int32)
    d = runtime.ProgramDesc(len(ranks), keep[0].ctypes.data_as(i32), keep[1].ctypes.data_as(i32),
                            vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(tokens),
                            keep[2].ctypes.data_as(i32), len(gsize), keep[3].ctypes.data_as(i32),
                            keep[4].ctypes.data_as(i32))
    return d, keep, vals


@pytest.mark.parametrize("case", ["empty", "bad_token", "join_underflow", "dup_group", "negative", "two_roots"])
def test_create_rejects_invalid_programs(lib, case):
    one = [1.0, 1.0]
    if case == "empty":
        d, *_ = _desc([], [], [], [])
    elif case == "bad_token":
        d, *_ = _desc([1], [0], one, [5])
    elif case == "join_underflow":
        d, *_ = _desc([1], [0], one, [0, -1])
    elif case == "dup_group":
        d, *_ = _desc([1, 1], [0, 0], one + one, [0, 1, -1], gsize=[1, 1], gedges=[0, 0])
    elif case == "negative":
        d, *_ = _desc([1, 1], [0, 0], [1.0, -1.0, 1.0, 1.0], [0, 1, -1])
    else:
        d, *_ = _desc([1, 1], [0, 1], one + one, [0, 1])
    h = ctypes.c_void_p()
    st = lib.togb_program_create(ctypes.byref(d), 0, ctypes.byref(h))
    assert st in (runtime.ERR_INVALID, runtime.ERR_UNSUPPORTED)
    assert not h.value
    assert lib.togb_last_error()


def test_tensordot_rejects_bad_axes(lib):
    a = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    axes = np.array([3], dtype=np.int32)
    st = lib.togb_tensordot_f64(a, 2, a, 2, 1, axes.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                axes.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), a, None)
    assert st == runtime.ERR_INVALID


def test_set_leaves_validates_before_touching_a_device(lib):
    """togb_program_set_leaves: null arguments are invalid, and a host-only
    program (no leaves on a device) is refused without any CUDA call."""
    from tensororder_gb300.program import Leaf, Program

    prog = Program([Leaf([0], "var", w_neg=0.4, w_pos=0.6), Leaf([0], "var", w_neg=0.5, w_pos=0.5)],
                   [0, 1, -1]).validate()
    hp = runtime.HostProgram(prog)
    specs, values = runtime._leaf_specs(prog.leaves)
    try:
        assert lib.togb_program_set_leaves(None, specs, None, 0, None) == runtime.ERR_INVALID
        assert lib.togb_program_set_leaves(hp._h, None, None, 0, None) == runtime.ERR_INVALID
        assert lib.togb_program_set_leaves(hp._h, specs, None, 0, None) == runtime.ERR_UNSUPPORTED
    finally:
        hp.close()
