"""The ``--tensor_library`` plugin: TensorOrder's Execution stage on a GB300.

Mirrors the reference's backend interface (duck-typed, as ``tensororder.py``
and ``execution.py`` use it): ``add_argument``, ``get_entry_size``,
``create_tensor``, ``tensordot``, ``contract``, ``contract_sliced``, ``warm``
(``tensor_apis/base_api.py:8-28``, ``tensor_apis/numpy_apis.py:4-65``,
``tensor_apis/tensorflow_apis.py:51-133``).

* ``gb300``       -- plain form: FP64 storage and arithmetic.
* ``gb300-split`` -- chosen form: FP32 storage with per-slice power-of-two
  exponents, FP64 only in the compensated slice sum.

``--entry_type`` picks the form as the reference's backends pick their dtype
(``numpy_apis.py:13-27``, ``tensorflow_apis.py:64-80``): ``float64`` keeps the
library's form, ``float32`` and ``float16`` take the split form (FP32 storage,
at least float16's range and precision), ``int`` and ``uint`` take the int
form (64-bit words, sums and products modulo 2^64, as numpy's int64 and
uint64 tensors wrap; the count is a numpy int64 or uint64 scalar).
``bigint`` (numpy object arrays of Python integers) gives the exact count as a
Python int, recovered from the int form's count modulo 2^64 and residue-form
counts modulo primes below 2^28 (:mod:`tensororder_gb300.exact`); networks
with non-integer leaf values give the plain FP64 count as a Python float, as
the reference's object arithmetic turns floating there.

``contract_sliced`` is the hot path.  It flattens the plan
(:func:`tensororder_gb300.program.from_plan`), hands it to libtogb and runs the
slices as a sequence of calls of bounded device time (about
``max_call_seconds`` each, sized from the measured time of the previous call).
After queueing a call it waits by polling a CUDA event from Python, so the
reference's SIGALRM timeout (``util.py:32-39`` raises ``TimeoutError`` from
the signal handler) fires mid-count, with at most one call's work left on the
device.  A device allocation failure raises the reference's
``OutOfMemoryError`` (``base_api.py:4``), whose handler in ``execution.py:134-142``
re-slices the plan and retries.  Nothing here falls back to a CPU path: if the
CUDA library or device is missing the call fails.
"""
from __future__ import annotations

import time

import numpy as np

from . import exact
from . import program as _program
from . import runtime


class OutOfMemoryError(Exception):
    """Stand-in for ``tensor_network.OutOfMemoryError`` until :func:`register`
    binds the reference's class."""


_OOM = OutOfMemoryError


class GB300API:
    """Execution backend; ``mode`` is ``runtime.MODE_F64``, ``runtime.MODE_SPLIT``
    or ``runtime.MODE_INT64``."""

    slices_per_call = 1 << 14  # upper bound on slices queued by one C call
    max_call_seconds = 0.25    # target device time of one call (timeout granularity)
    # device rate for sizing the first call before any has been timed (FLOP/s)
    _first_call_rate = {runtime.MODE_F64: 1.0e12, runtime.MODE_SPLIT: 5.0e13, runtime.MODE_INT64: 3.0e11,
                        runtime.MODE_MOD: 1.5e11}
    # numpy type of the int form's count, by entry type
    _word_types = {"int": np.int64, "uint": np.uint64}

    # Keep the last lowered program: a later count of the same network (same
    # tree, slice groups, leaf axes and kinds) only uploads its leaves.
    cache_programs = True

    def __init__(self, mode=runtime.MODE_F64, device=0):
        self._mode = mode
        self._word_type = np.int64  # the int form's count type
        self._bigint = False        # exact counts through the int forms
        self._device = device
        self._thread_limit = None
        self.last_program = None
        self._cached = None  # (structure key, DeviceProgram)

    # -- configuration (numpy_apis.py:13-34) --------------------------------
    def add_argument(self, key, value):
        if key == "entry_type":
            if value not in ("float64", "float32", "float16", "bigint") and value not in self._word_types:
                raise ValueError("Unknown gb300 type %s" % value)
            self._bigint = value == "bigint"
            if value in ("float32", "float16"):
                self._mode = runtime.MODE_SPLIT
            elif value in self._word_types:
                self._mode = runtime.MODE_INT64
                self._word_type = self._word_types[value]
            return
        if key == "thread_limit":
            # Host thread cap of the numpy backend; the device path has no host
            # compute threads to limit.
            self._thread_limit = value
            return
        raise ValueError("Invalid argument " + str(key) + " for selected tensor_library")

    def get_entry_size(self):
        return 4 if self._mode == runtime.MODE_SPLIT and not self._bigint else 8

    # -- tensor primitives ---------------------------------------------------
    def create_tensor(self, shape, default_value=None):
        """Host tensor for ``Tensor.build`` (leaves are built on the host and
        uploaded once per program)."""
        if default_value is None:
            return np.empty(shape, dtype=np.float64)
        return np.full(shape, default_value, dtype=np.float64)

    def tensordot(self, a, b, axes):
        """``np.tensordot`` on the device; numpy inputs are uploaded.  The
        result is a float64 CUDA tensor, or for the ``int`` / ``uint`` entry
        types an int64 one (64-bit words, sums and products modulo 2^64, as
        numpy's int64 and uint64 tensordot gives them)."""
        import torch

        dev = torch.device("cuda", self._device)
        words = self._mode == runtime.MODE_INT64 and not self._bigint

        def as_dev(x):
            if words:
                if isinstance(x, torch.Tensor):
                    return x.to(device=dev, dtype=torch.int64)
                v = np.asarray(x)
                if v.dtype.kind == "f":
                    v = v.astype(np.int64)  # toward zero, numpy's cast
                return torch.as_tensor(np.ascontiguousarray(v.astype(np.uint64, copy=False).view(np.int64)),
                                       device=dev)
            if isinstance(x, torch.Tensor):
                return x.to(device=dev, dtype=torch.float64)
            return torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev)

        if words:
            return runtime.tensordot_i64(as_dev(a), as_dev(b), axes)
        return runtime.tensordot_f64(as_dev(a), as_dev(b), axes)

    def warm(self):
        """Load the library and create the CUDA context with one tiny contraction."""
        import torch

        a = torch.full((2,), 2.0, dtype=torch.float64, device=torch.device("cuda", self._device))
        runtime.tensordot_f64(a, a, ([0], [0]))
        torch.cuda.synchronize(self._device)

    # -- contraction ---------------------------------------------------------
    def contract(self, network, contraction_tree):
        """Contract one (already sliced or unsliced) network along a tree, as
        ``NumpyAPI.contract`` (``numpy_apis.py:45-55``) does."""

        class _Plan:
            pass

        plan = _Plan()
        plan.network, plan.tree, plan.groups_to_slice = network, contraction_tree, []
        return np.asarray(self._run(_program.from_plan(plan), None))

    def contract_sliced(self, execution_plan, num_slice_limit=None):
        """Sum of the contractions of every slice of the plan
        (``base_api.py:17-28``); ``num_slice_limit`` keeps a prefix in
        ``itertools.product`` order."""
        value = self._run(_program.from_plan(execution_plan), num_slice_limit)
        return value[()] if np.ndim(value) == 0 else value

    def contract_program(self, prog, num_slice_limit=None):
        """Same as ``contract_sliced`` for an already flattened program."""
        value = self._run(prog, num_slice_limit)
        return value[()] if np.ndim(value) == 0 else value

    def _stream(self):
        import torch

        return torch.cuda.current_stream(self._device)

    @staticmethod
    def _wait(stream):
        """Wait for the work queued on ``stream`` while returning to the
        interpreter between polls, so a pending signal handler (the
        reference's SIGALRM timeout) runs and may raise."""
        import torch

        ev = torch.cuda.Event()
        ev.record(stream)
        t0 = time.perf_counter()
        while not ev.query():
            if time.perf_counter() - t0 > 2e-3:
                time.sleep(2e-4)

    @staticmethod
    def _structure_key(prog):
        """What the lowering depends on: the tree, the slice groups and every
        leaf's axes and kind (clause, variable or dense) -- not the weights."""
        def kind(l):
            return 1 if (l.kind == "or" and l.rank <= 30) else (2 if l.kind == "var" else 0)
        return (tuple(prog.postorder), tuple(tuple(g) for g in prog.slice_groups),
                tuple((kind(l), tuple(l.axes)) for l in prog.leaves))

    def _program(self, prog, stream):
        """The device program for ``prog``: the cached one with ``prog``'s
        leaves uploaded when the structure matches, else a new one."""
        if not self.cache_programs:
            return runtime.DeviceProgram(prog, self._device)
        key = self._structure_key(prog)
        if self._cached is not None and self._cached[0] == key:
            dp = self._cached[1]
            dp.set_leaves(prog, stream)
            return dp
        if self._cached is not None:  # release its device memory before lowering the next
            self._cached[1].close()
            self._cached = None
        dp = runtime.DeviceProgram(prog, self._device)
        self._cached = (key, dp)
        return dp

    def _run(self, prog, num_slice_limit):
        n = prog.num_slices if num_slice_limit is None else min(prog.num_slices, int(num_slice_limit))
        try:
            stream = self._stream()
            dp = self._program(prog, stream)
            self.last_program = dp
            if self._bigint:
                return self._exact(prog, dp, n, stream)
            self._count(dp, self._mode, n, stream)
            if self._mode == runtime.MODE_INT64:
                return dp.result_words(stream, self._word_type)
            return dp.result(stream)
        except runtime.DeviceOutOfMemory as exc:
            raise _OOM(str(exc))

    def _count(self, dp, mode, n, stream):
        """Reset the accumulator and add slices [0, n) in ``mode``, as calls of
        bounded device time with a wait after each."""
        dp.reset(stream)
        ws = dp.allocate_workspace(mode, max(n, 1))
        # First call sized from the FLOP count, later ones from the measured
        # time per slice of the previous call.
        per_slice = max(float(dp.info.flops_per_slice), 1.0) / self._first_call_rate[mode]
        s = 0
        while s < n:
            k = int(min(self.slices_per_call, max(1, self.max_call_seconds / max(per_slice, 1e-9))))
            e = min(n, s + k)
            t0 = time.perf_counter()
            dp.run(mode, s, e, workspace=ws, stream=stream)
            self._wait(stream)
            per_slice = (time.perf_counter() - t0) / (e - s)
            s = e

    def _exact(self, prog, dp, n, stream):
        """The ``bigint`` count: exact Python integers from the int forms'
        residues, or the plain FP64 count (Python floats) when a leaf value is
        not an integer."""
        if not exact.integer_leaves(prog):
            self._count(dp, runtime.MODE_F64, n, stream)
            return dp.result(stream).astype(object)
        # Leaf values are non-negative (program creation refuses others), so
        # the split form's count bounds the count to about 1e-6.
        self._count(dp, runtime.MODE_SPLIT, n, stream)
        bound = float(np.max(np.abs(dp.result(stream))))
        moduli = exact.moduli_for(bound * (1.0 + 1e-4) + 1.0)
        self._count(dp, runtime.MODE_INT64, n, stream)
        words = dp.result_words(stream, np.uint64)
        residues = []
        for p in moduli:
            dp.set_modulus(p)
            self._count(dp, runtime.MODE_MOD, n, stream)
            residues.append(dp.result_words(stream, np.uint64).reshape(-1))
        out = np.empty(words.size, dtype=object)
        for i, w in enumerate(words.reshape(-1)):
            out[i] = exact.combine(int(w), [int(r[i]) for r in residues], moduli)
        return out.reshape(words.shape)


class GB300SplitAPI(GB300API):
    def __init__(self, device=0):
        super().__init__(mode=runtime.MODE_SPLIT, device=device)


GB300_APIS = {
    "gb300": GB300API,
    "gb300-split": GB300SplitAPI,
}


def register(all_apis=None):
    """Add the plugins to the reference's ``tensor_network.ALL_APIS``.

    ``--tensor_library`` is resolved through ``util.TaggedChoice`` over that
    live dict (``util.py:249-252``), so registering before the CLI runs is all
    the integration needed; no reference file is edited.
    """
    global _OOM
    import tensor_network

    _OOM = tensor_network.OutOfMemoryError
    target = tensor_network.ALL_APIS if all_apis is None else all_apis
    target.update(GB300_APIS)
    return target
