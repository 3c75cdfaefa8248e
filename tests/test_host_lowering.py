"""Host-only lowering (no GPU): the launch plan of a count.

The slice-invariant joins of a program run as fused lists of thread-per-output
joins plus single launches of the other joins; a count is that phase, then per
chunk of slices the slice-base update, every per-slice join and the root
reduction.  `togb_program_launch_count` of a host-only program gives the plan a
run would queue with every slice in one chunk."""
import ctypes
import gzip
import json
import os

import pytest

from conftest import ROOT, golden_names, load_golden
from tensororder_gb300 import runtime
from tensororder_gb300.program import Program


def launch_plan(prog, mode):
    hp = runtime.HostProgram(prog)
    try:
        out = ctypes.c_int64()
        runtime.check(runtime.lib().togb_program_launch_count(hp._h, int(mode), ctypes.byref(out)))
        return out.value, int(hp.info.num_joins_once), int(hp.info.num_launches)
    finally:
        hp.close()


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
def test_launch_count_of_golden_plans(name, mode):
    prog = Program.from_dict(load_golden(name)["program"])
    launches, once, per_and_root = launch_plan(prog, mode)
    per_chunk = per_and_root + 1  # slice base, per-slice joins, root
    if once == 0:
        assert launches == per_chunk
    else:
        assert 1 <= launches - per_chunk <= min(once, 4)


@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
def test_n220_slice_invariant_phase_is_two_launches(mode):
    """360 thread-per-output joins in one fused list and one GEMM-shaped join."""
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc220_s10.json.gz"), "rt") as f:
        prog = Program.from_dict(json.load(f)["program"])
    launches, once, per_and_root = launch_plan(prog, mode)
    assert once == 361
    assert launches == 2 + per_and_root + 1


@pytest.mark.parametrize("m,n,k,plain,split", [
    (5, 14, 5, 1, 3), (14, 5, 5, 1, 3), (5, 5, 4, 1, 3), (6, 6, 4, 1, 3),  # GEMM-classed: M, N >= 32, K >= 16
    (4, 14, 5, 0, 0), (5, 14, 3, 0, 0), (12, 2, 1, 0, 0),                   # thread-per-output
])
def test_gemm_classification(m, n, k, plain, split):
    """A join of two intermediates is GEMM-classed when M, N >= 32 and K >= 16:
    the plain form runs it on the tiled kernel (1), the split form on the
    tensor cores (3); smaller ones stay on the thread-per-output kernel (0)."""
    import sys

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_gpu_gemm_joins import make_program

    prog = make_program(7 + m + n + k, m, n, k)
    hp = runtime.HostProgram(prog)
    try:
        root = prog.num_joins - 1
        got = (int(hp.joins(runtime.MODE_F64)[root][3]), int(hp.joins(runtime.MODE_SPLIT)[root][3]))
        mnk = sorted((int(x) for x in hp.joins(runtime.MODE_SPLIT)[root][:2]))
    finally:
        hp.close()
    assert mnk == sorted((m, n))
    assert got == (plain, split)


@pytest.mark.parametrize("name", golden_names())
def test_int_forms_lower_like_the_plain_form(name):
    """The int form and the residue form share the plain form's 8-byte layout
    and kernels (no tensor-core kernel); the residue form describes and
    counts launches before any modulus is set (its Barrett constant is filled
    only once a modulus exists), and both forms need as much workspace as
    the plain form."""
    prog = Program.from_dict(load_golden(name)["program"])
    hp = runtime.HostProgram(prog)
    try:
        plain = hp.joins(runtime.MODE_F64)
        for mode in (runtime.MODE_INT64, runtime.MODE_MOD):
            assert (hp.joins(mode) == plain).all()
            for j in range(len(plain)):
                assert not hp.kernel_allowed(mode, j, 3)
                assert hp.kernel_allowed(mode, j, 1)
                assert "kernel %d" % plain[j][3] in hp.describe(mode, j)
            assert hp.info.workspace_per_slice[mode] == hp.info.workspace_per_slice[runtime.MODE_F64]
            assert hp.info.workspace_fixed[mode] == hp.info.workspace_fixed[runtime.MODE_F64]
        assert launch_plan(prog, runtime.MODE_MOD) == launch_plan(prog, runtime.MODE_F64)
        assert launch_plan(prog, runtime.MODE_INT64) == launch_plan(prog, runtime.MODE_F64)
    finally:
        hp.close()


def test_unknown_modes_are_rejected():
    hp = runtime.HostProgram(Program.from_dict(load_golden("vc60_s4")["program"]))
    try:
        for mode in (-1, 4, 99):
            with pytest.raises(runtime.TogbError):
                hp.joins(mode)
            with pytest.raises(runtime.TogbError):
                hp.describe(mode, 0)
            with pytest.raises(runtime.TogbError):
                hp.kernel_allowed(mode, 0, 0)
        for bad in (0, 1, 1 << 28):
            with pytest.raises(runtime.TogbError):
                runtime.check(runtime.lib().togb_program_set_modulus(hp._h, bad))
        runtime.check(runtime.lib().togb_program_set_modulus(hp._h, 268435399))
    finally:
        hp.close()
