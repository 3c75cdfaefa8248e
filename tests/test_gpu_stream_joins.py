"""Joins of a long intermediate with a tiny leaf -- the joins the split form
runs on the streaming thread-per-quad kernel.  X (ranks 10-14) is the outer
product of two seeded dense leaves; the root join contracts it with a dense
leaf Y of at most 16 entries over k <= 2 shared edges (or k = 3 against a
single free edge).  The cases are chosen so
that X's two lowest m bits are either its two lowest address bits or lie just
above its k bits (the two operand layouts the streaming kernel reads), which
the host-only lowering confirms without a GPU.  Sliced cases put the slice
edges on Y and on X (per-slice X), on Y alone (slice-invariant X, computed
once and read by every slice) or on X alone (slice-invariant leaf Y).  The
same generator gives the short-K joins with large outputs that run on the
staged kernel.  Tolerances: 1e-12 (plain), 1e-6 (split),
relative to the largest entry."""
import numpy as np
import pytest

from oracle import contract as oracle
from tensororder_gb300 import runtime
from tensororder_gb300.program import Leaf, Program


def make_program(seed, m, k, n, slices=0, where="xy"):
    """Slice edges on X's first leaf and on Y (``xy``), on Y only (``y``:
    slice-invariant X, Y the product of two leaves sharing them) or on X only
    (``x``: X's two leaves share them, Y a slice-invariant leaf)."""
    rng = np.random.default_rng(seed)
    fa = list(range(m))
    kk = list(range(m, m + k))
    fb = list(range(m + k, m + k + n))
    xa = [int(e) for e in rng.permutation(fa + kk)]
    ya = [int(e) for e in rng.permutation(kk + fb)]
    cut = len(xa) // 2
    sl = [m + k + n + g for g in range(slices)]
    if where == "xy":
        leaves = [Leaf(xa[:cut] + sl, "dense"), Leaf(xa[cut:], "dense"), Leaf(ya + sl, "dense")]
        post = [0, 1, -1, 2, -1]
    elif where == "x":
        leaves = [Leaf(xa[:cut] + sl, "dense"), Leaf(xa[cut:] + sl, "dense"), Leaf(ya, "dense")]
        post = [0, 1, -1, 2, -1]
    else:
        half = len(ya) // 2
        leaves = [Leaf(xa[:cut], "dense"), Leaf(xa[cut:], "dense"), Leaf(ya[:half] + sl, "dense"),
                  Leaf(ya[half:] + sl, "dense")]
        post = [0, 1, -1, 2, 3, -1, -1]
    for leaf in leaves:
        leaf.values = rng.uniform(0.5, 1.5, size=(2,) * leaf.rank)
    return Program(leaves, post, [[e] for e in sl]).validate()


def stream_layout(prog, join):
    """'mfast' / 'kfast' when the join's A operand has one of the two streaming
    layouts and its output is natural; None otherwise."""
    hp = runtime.HostProgram(prog)
    try:
        txt = hp.describe(runtime.MODE_SPLIT, join)
    finally:
        hp.close()
    head = txt.splitlines()[0].split()
    natural = int(head[head.index("c_natural") + 1])
    mb, nb, kb = (int(x) for x in head[3:6])
    so = sk = None
    a_lo = False
    for line in txt.splitlines():
        t = line.split()
        if t[:2] == ["A", "s_outer"]:
            so = [int(x) for x in t[2:]]
        if t[:2] == ["A", "s_k"]:
            sk = [int(x) for x in t[2:]]
        if t[:2] == ["A", "leaf"]:
            a_lo = int(t[2]) == 1
    if not natural or a_lo or kb > 3 or (kb == 3 and nb > 0) or (1 << (nb + kb)) > 16 or mb < 2:
        return None
    K = 1 << kb
    if so[:2] == [1, 2]:
        return "mfast"
    if kb >= 1 and so[:2] == [K, 2 * K] and sk == [1 << j for j in range(kb)]:
        return "kfast"
    return None


# (seed, m, k, n, slices, where, layout)
CASES = [
    (0, 12, 1, 2, 0, "xy", "mfast"), (13, 12, 1, 2, 0, "xy", "kfast"), (0, 13, 2, 1, 0, "xy", "mfast"),
    (0, 12, 0, 4, 0, "xy", "mfast"), (1, 11, 2, 2, 0, "xy", "mfast"), (39, 11, 2, 2, 0, "xy", "kfast"),
    (4, 14, 1, 3, 0, "xy", "kfast"), (2, 14, 1, 3, 0, "xy", "mfast"), (3, 10, 2, 0, 0, "xy", "mfast"),
    (1, 12, 1, 2, 2, "xy", "mfast"), (32, 12, 1, 2, 2, "xy", "kfast"), (5, 13, 2, 1, 3, "xy", "mfast"),
    (6, 14, 1, 3, 2, "xy", "kfast"), (2, 12, 0, 4, 2, "xy", "mfast"),
    (0, 12, 1, 2, 3, "y", "mfast"), (13, 12, 1, 2, 2, "y", "kfast"), (4, 14, 1, 3, 3, "y", "kfast"),
    (1, 13, 2, 1, 2, "y", "mfast"), (3, 12, 0, 4, 2, "y", "mfast"),
    # fewer than 32 x U quads of m per slice: the per-quad kernel (the cases
    # above have enough for the warp-block kernel)
    (0, 8, 1, 2, 0, "xy", "mfast"), (3, 8, 1, 2, 0, "xy", "kfast"), (0, 7, 2, 1, 0, "xy", "mfast"),
    (44, 7, 2, 1, 0, "xy", "kfast"), (0, 6, 0, 3, 0, "xy", "mfast"), (12, 8, 2, 2, 0, "xy", "kfast"),
    (2, 7, 1, 3, 0, "xy", "mfast"),
    # K = 8 against a single column (N = 1)
    (0, 12, 3, 0, 0, "xy", "mfast"), (2, 13, 3, 0, 2, "xy", "mfast"), (0, 12, 3, 0, 2, "y", "mfast"),
    (1, 8, 3, 0, 2, "xy", "mfast"), (1, 7, 3, 0, 0, "xy", "mfast"), (24, 7, 3, 0, 0, "xy", "kfast"),
    (24, 7, 3, 0, 2, "y", "kfast"),
]


def _prog(case):
    seed, m, k, n, slices, where, _ = case
    return make_program(seed, m, k, n, slices, where)


@pytest.mark.parametrize("case", CASES)
def test_cases_have_the_streaming_layout(case):
    """Host-only lowering: the root join of every case has a streaming layout,
    and the library's own variant choice for it is the streaming kernel."""
    prog = _prog(case)
    root = prog.postorder.count(-1) - 1
    assert stream_layout(prog, root) == case[-1]
    assert _variant(prog, root) == ("stream" if case[-1] == "mfast" else "stream_kfast")


# Short-K joins whose output tiles reuse operand rows: the staged kernel,
# including the orders that keep a slice-invariant operand's rows staged.
STAGED = [
    (0, 12, 2, 7, 2, "y", "staged"), (1, 12, 2, 7, 2, "x", "staged"), (2, 12, 2, 7, 2, "xy", "staged"),
    (3, 9, 2, 9, 3, "y", "staged"), (4, 9, 2, 9, 2, "x", "staged"), (5, 11, 3, 5, 2, "x", "staged"),
    (6, 8, 0, 8, 2, "y", "staged"), (7, 10, 1, 6, 0, "xy", "staged"),
    # 64 slices: enough tiles for the 2^13 / 2^14-address tiles
    (8, 12, 2, 7, 6, "y", "staged"), (9, 9, 2, 9, 6, "x", "staged"), (10, 11, 3, 5, 6, "xy", "staged"),
]


def _variant(prog, join):
    hp = runtime.HostProgram(prog)
    try:
        head = hp.describe(runtime.MODE_SPLIT, join).splitlines()[0].split()
    finally:
        hp.close()
    return head[head.index("variant") + 1]


@pytest.mark.parametrize("case", STAGED)
def test_staged_cases_take_the_staged_kernel(case):
    prog = _prog(case)
    assert _variant(prog, prog.postorder.count(-1) - 1) == "staged"


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES + STAGED)
@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)])
def test_stream_join(case, mode, tol, cuda):
    prog = _prog(case)
    want = sum(oracle.contract(prog, s)[0] for s in range(prog.num_slices))
    dp = runtime.DeviceProgram(prog)
    dp.reset()
    dp.run(mode)
    got = dp.result()
    dp.close()
    assert got.shape == want.shape
    assert np.abs(got - want).max() <= tol * np.abs(want).max()
