"""ctypes bindings of ``libtogb.so`` (the C ABI declared in ``include/togb.h``).

PyTorch is used only for device memory and streams: workspaces are
``torch.empty(..., dtype=torch.uint8, device="cuda")`` buffers and work is
queued on ``torch.cuda.current_stream()``.  No compute goes through torch.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from .program import Program

MODE_F64 = 0
MODE_SPLIT = 1
MODE_INT64 = 2  # 64-bit integer words, sums and products modulo 2^64
MODE_MOD = 3    # residues modulo the program's modulus (DeviceProgram.set_modulus)

OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_UNSUPPORTED, ERR_TIMEOUT = range(6)

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)


class ProgramDesc(ctypes.Structure):
    _fields_ = [
        ("num_leaves", ctypes.c_int32),
        ("leaf_rank", _i32p),
        ("leaf_axes", _i32p),
        ("leaf_values", _f64p),
        ("num_tokens", ctypes.c_int32),
        ("postorder", _i32p),
        ("num_groups", ctypes.c_int32),
        ("group_size", _i32p),
        ("group_edges", _i32p),
    ]


class ProgramInfo(ctypes.Structure):
    _fields_ = [
        ("num_slices", ctypes.c_int64),
        ("num_joins", ctypes.c_int32),
        ("max_rank", ctypes.c_int32),
        ("root_rank", ctypes.c_int32),
        ("num_launches", ctypes.c_int32),
        ("flops_per_slice", ctypes.c_double),
        ("bytes_per_slice_f64", ctypes.c_double),
        ("workspace_per_slice", ctypes.c_int64 * 4),
        ("workspace_fixed", ctypes.c_int64 * 4),
        ("num_joins_once", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("flops_once", ctypes.c_double),
        ("bytes_once_f64", ctypes.c_double),
    ]


class LeafSpec(ctypes.Structure):
    """togb_leaf_spec: a clause or variable leaf by its parameters."""

    _fields_ = [
        ("kind", ctypes.c_int32),
        ("output_index", ctypes.c_int32),
        ("positive", ctypes.c_uint32),
        ("pad_", ctypes.c_int32),
        ("w_neg", ctypes.c_double),
        ("w_pos", ctypes.c_double),
    ]


LEAF_DENSE, LEAF_CLAUSE, LEAF_VARIABLE = 0, 1, 2


class TogbError(RuntimeError):
    """A failed call into libtogb; ``status`` is the togb_status code."""

    def __init__(self, status, message):
        super().__init__("libtogb status %d: %s" % (status, message))
        self.status = status


class DeviceOutOfMemory(TogbError):
    """Device memory did not suffice (TOGB_ERR_OOM or a failed torch allocation)."""


_lib = None

EXPORTS = [
    "togb_version", "togb_last_error", "togb_program_create", "togb_program_info_get",
    "togb_program_reset", "togb_program_run", "togb_program_result", "togb_program_set_timing",
    "togb_program_join_times", "togb_program_destroy", "togb_tensordot_f64", "togb_probe_peak",
    "togb_contract_static_f64", "togb_program_joins", "togb_program_set_kernel", "togb_program_kernel_allowed",
    "togb_mlp_param_count", "togb_mlp_scratch_floats", "togb_mlp_forward", "togb_mlp_loss_grad", "togb_mlp_adam",
    "togb_batch_create", "togb_batch_run", "togb_batch_results", "togb_batch_destroy",
    "togb_program_create_host", "togb_program_describe", "togb_program_create_compact",
    "togb_program_launch_count", "togb_program_set_wait_limit", "togb_program_set_leaves",
    "togb_program_result_u64", "togb_program_set_modulus", "togb_tensordot_i64",
]

KERNEL_NAMES = {0: "direct", 1: "tiled", 2: "reduce", 3: "tensor"}

STATIC_SCRATCH_BYTES = 32 << 20


def library_path():
    return _build.LIB


def lib():
    """Load ``libtogb.so``; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError("libtogb.so is missing (%s); run tensororder_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    c_void = ctypes.c_void_p
    L.togb_version.restype = ctypes.c_int
    L.togb_last_error.restype = ctypes.c_char_p
    L.togb_program_create.argtypes = [ctypes.POINTER(ProgramDesc), ctypes.c_int, ctypes.POINTER(c_void)]
    L.togb_program_info_get.argtypes = [c_void, ctypes.POINTER(ProgramInfo)]
    L.togb_program_reset.argtypes = [c_void, c_void]
    L.togb_program_run.argtypes = [c_void, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, c_void, ctypes.c_size_t, c_void]
    L.togb_program_result.argtypes = [c_void, c_void, _f64p, _f64p, ctypes.c_int64]
    L.togb_program_result_u64.argtypes = [c_void, c_void, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int64]
    L.togb_program_set_modulus.argtypes = [c_void, ctypes.c_uint64]
    L.togb_program_set_timing.argtypes = [c_void, ctypes.c_int]
    L.togb_program_join_times.argtypes = [c_void, ctypes.POINTER(ctypes.c_float), ctypes.c_int32]
    L.togb_program_destroy.argtypes = [c_void]
    L.togb_program_destroy.restype = None
    L.togb_tensordot_f64.argtypes = [c_void, ctypes.c_int32, c_void, ctypes.c_int32, ctypes.c_int32,
                                     _i32p, _i32p, c_void, c_void]
    L.togb_tensordot_i64.argtypes = L.togb_tensordot_f64.argtypes
    L.togb_probe_peak.argtypes = [ctypes.c_int, c_void, ctypes.POINTER(ctypes.c_double)]
    L.togb_contract_static_f64.argtypes = [ctypes.POINTER(ProgramDesc), c_void, c_void, c_void]
    L.togb_program_joins.argtypes = [c_void, ctypes.c_int, _i32p, ctypes.c_int32]
    L.togb_program_launch_count.argtypes = [c_void, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    L.togb_program_set_kernel.argtypes = [c_void, ctypes.c_int, ctypes.c_int32, ctypes.c_int32]
    L.togb_program_set_wait_limit.argtypes = [c_void, ctypes.c_int64]
    L.togb_program_set_leaves.argtypes = [c_void, ctypes.POINTER(LeafSpec), _f64p, ctypes.c_int64, c_void]
    L.togb_program_kernel_allowed.argtypes = [c_void, ctypes.c_int, ctypes.c_int32, ctypes.c_int32, _i32p]
    L.togb_batch_create.argtypes = [ctypes.POINTER(c_void), ctypes.c_int32, ctypes.c_int, ctypes.POINTER(c_void),
                                    ctypes.POINTER(ctypes.c_size_t), ctypes.c_int32, ctypes.POINTER(c_void)]
    L.togb_batch_run.argtypes = [c_void, c_void]
    L.togb_program_create_host.argtypes = [ctypes.POINTER(ProgramDesc), ctypes.POINTER(c_void)]
    L.togb_program_create_compact.argtypes = [ctypes.POINTER(ProgramDesc), ctypes.POINTER(LeafSpec), ctypes.c_int,
                                              ctypes.POINTER(c_void)]
    L.togb_program_describe.argtypes = [c_void, ctypes.c_int, ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t]
    L.togb_batch_results.argtypes = [c_void, c_void, _f64p, ctypes.c_int32]
    L.togb_batch_destroy.argtypes = [c_void]
    L.togb_batch_destroy.restype = None
    for name in EXPORTS:
        if name not in ("togb_version", "togb_last_error", "togb_program_destroy", "togb_batch_destroy") \
                and not name.startswith("togb_mlp"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def check(status):
    if status != OK:
        msg = lib().togb_last_error().decode(errors="replace")
        if status == ERR_OOM:
            raise DeviceOutOfMemory(status, msg)
        raise TogbError(status, msg)


def _stream_handle(stream):
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _leaf_specs(leaves):
    """togb_leaf_spec records of ``leaves`` and the dense leaves' values
    (concatenated in leaf order, or None when no leaf is dense)."""
    specs = (LeafSpec * max(1, len(leaves)))()
    vals = []
    for i, l in enumerate(leaves):
        sp = specs[i]
        if l.kind == "or" and l.rank <= 30:
            sp.kind = LEAF_CLAUSE
            sp.output_index = -1 if l.output_index is None else int(l.output_index)
            sp.positive = sum(1 << a for a, pos in enumerate(l.positive) if pos)
        elif l.kind == "var":
            sp.kind = LEAF_VARIABLE
            sp.w_neg, sp.w_pos = float(l.w_neg), float(l.w_pos)
        else:
            sp.kind = LEAF_DENSE
            vals.append(l.parent().ravel())
    values = np.ascontiguousarray(np.concatenate(vals), dtype=np.float64) if vals else None
    return specs, values


class _Desc:
    """A togb_program_desc with the arrays it points into kept alive.

    ``values``: "all" concatenates every leaf's dense values (togb_program_create),
    "dense" only the dense leaves' (togb_program_create_compact, with ``specs``
    describing the clause and variable leaves), None none at all."""

    def __init__(self, program: Program, values="all"):
        leaves = program.leaves
        self.ranks = np.array([l.rank for l in leaves], dtype=np.int32)
        self.axes = np.array([a for l in leaves for a in l.axes] or [0], dtype=np.int32)
        self.specs = None
        if values == "all":
            vals = [l.parent().ravel() for l in leaves]
            self.values = np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1), dtype=np.float64)
        elif values == "dense":
            self.specs, self.values = _leaf_specs(leaves)
        else:
            self.values = None
        self.tokens = np.array(program.postorder, dtype=np.int32)
        self.gsize = np.array([len(g) for g in program.slice_groups] or [0], dtype=np.int32)
        self.gedges = np.array([e for g in program.slice_groups for e in g] or [0], dtype=np.int32)
        self.desc = ProgramDesc(
            len(leaves), self.ranks.ctypes.data_as(_i32p), self.axes.ctypes.data_as(_i32p),
            self.values.ctypes.data_as(_f64p) if self.values is not None else None, len(self.tokens),
            self.tokens.ctypes.data_as(_i32p), len(program.slice_groups), self.gsize.ctypes.data_as(_i32p),
            self.gedges.ctypes.data_as(_i32p))


class HostProgram:
    """A program lowered and planned on the host only, for inspection
    (``togb_program_create_host``): joins, allowed kernels, layouts."""

    def __init__(self, program: Program):
        self.program = program
        self._d = _Desc(program, values=None)
        handle = ctypes.c_void_p()
        check(lib().togb_program_create_host(ctypes.byref(self._d.desc), ctypes.byref(handle)))
        self._h = handle
        info = ProgramInfo()
        check(lib().togb_program_info_get(self._h, ctypes.byref(info)))
        self.info = info

    def joins(self, mode):
        n = int(self.info.num_joins)
        out = np.zeros((max(n, 1), 5), dtype=np.int32)
        check(lib().togb_program_joins(self._h, int(mode), out.ctypes.data_as(_i32p), n))
        return out[:n]

    def describe(self, mode, join):
        buf = ctypes.create_string_buffer(8192)
        check(lib().togb_program_describe(self._h, int(mode), int(join), buf, 8192))
        return buf.value.decode()

    def kernel_allowed(self, mode, join, kernel):
        out = ctypes.c_int32()
        check(lib().togb_program_kernel_allowed(self._h, int(mode), int(join), int(kernel), ctypes.byref(out)))
        return bool(out.value)

    def close(self):
        if getattr(self, "_h", None):
            lib().togb_program_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceProgram:
    """A program lowered and planned by libtogb, with its leaves on the device."""

    def __init__(self, program: Program, device: int = 0, leaves: str = "device"):
        """``leaves="device"``: clause and variable leaves are described by
        their parameters and built on the device, only dense leaves' values are
        uploaded (togb_program_create_compact).  ``leaves="host"``: every
        leaf's dense values are built here and uploaded (togb_program_create)."""
        self.program = program
        self.device = device
        handle = ctypes.c_void_p()
        if leaves == "device":
            self._d = _Desc(program, values="dense")
            self.h2d_bytes = (0 if self._d.values is None else self._d.values.nbytes * 2) + \
                ctypes.sizeof(LeafSpec) * len(program.leaves)
            check(lib().togb_program_create_compact(ctypes.byref(self._d.desc), self._d.specs, device,
                                                    ctypes.byref(handle)))
        elif leaves == "host":
            self._d = _Desc(program, values="all")
            self.h2d_bytes = self._d.values.nbytes * 2
            check(lib().togb_program_create(ctypes.byref(self._d.desc), device, ctypes.byref(handle)))
        else:
            raise ValueError("leaves must be 'device' or 'host'")
        self._h = handle
        info = ProgramInfo()
        check(lib().togb_program_info_get(self._h, ctypes.byref(info)))
        self.info = info
        self._workspace = None

    def set_leaves(self, program: Program, stream=None):
        """Upload the leaves of ``program`` -- the same network with other
        weights or clause polarities (leaf kinds, ranks, axes, tree and slice
        groups equal to this program's) -- and build them on the device,
        queued on ``stream``.  Only for programs created with
        ``leaves="device"``."""
        specs, values = _leaf_specs(program.leaves)
        n = 0 if values is None else int(values.size)
        vals = values.ctypes.data_as(_f64p) if values is not None else None
        check(lib().togb_program_set_leaves(self._h, specs, vals, n, _stream_handle(stream)))
        self.program = program
        self._leaf_data = (specs, values)  # kept alive while the copies are queued
        self.h2d_bytes = (0 if values is None else values.nbytes * 2) + ctypes.sizeof(LeafSpec) * len(program.leaves)

    @property
    def _values(self):
        """Every leaf's dense values concatenated (the layout the leaf arrays
        have on the device), built on the host on demand."""
        vals = [l.parent().ravel() for l in self.program.leaves]
        return np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1), dtype=np.float64)

    @property
    def num_slices(self):
        return int(self.info.num_slices)

    def workspace_bytes(self, mode, slices):
        return int(self.info.workspace_per_slice[mode]) * int(slices) + int(self.info.workspace_fixed[mode])

    def allocate_workspace(self, mode, slices, max_fraction=0.5):
        """A torch uint8 device buffer for up to ``slices`` slices per chunk,
        capped at ``max_fraction`` of free device memory (at least one slice)."""
        import torch

        per = int(self.info.workspace_per_slice[mode])
        free, _ = torch.cuda.mem_get_info(self.device)
        cap = max(1, int(free * max_fraction) // max(per, 1))
        n = max(1, min(int(slices), cap))
        want = self.workspace_bytes(mode, n)
        if self._workspace is not None and self._workspace.numel() >= want:
            return self._workspace
        self._workspace = None
        try:
            self._workspace = torch.empty(want, dtype=torch.uint8, device="cuda:%d" % self.device)
        except torch.cuda.OutOfMemoryError as e:
            raise DeviceOutOfMemory(ERR_OOM, str(e))
        return self._workspace

    def reset(self, stream=None):
        check(lib().togb_program_reset(self._h, _stream_handle(stream)))

    def run(self, mode, begin=0, end=None, workspace=None, stream=None):
        end = self.num_slices if end is None else end
        if workspace is None:
            ptr, nbytes = None, 0
        else:
            ptr, nbytes = workspace.data_ptr(), workspace.numel() * workspace.element_size()
        check(lib().togb_program_run(self._h, int(mode), int(begin), int(end), ctypes.c_void_p(ptr),
                                     ctypes.c_size_t(nbytes), _stream_handle(stream)))

    def result(self, stream=None):
        n = 1 << int(self.info.root_rank)
        out = np.zeros(n, dtype=np.float64)
        check(lib().togb_program_result(self._h, _stream_handle(stream), out.ctypes.data_as(_f64p), None, n))
        return out.reshape((2,) * int(self.info.root_rank))

    def set_modulus(self, modulus):
        """The residue form's modulus, in [2, 2^28)."""
        check(lib().togb_program_set_modulus(self._h, int(modulus)))

    def result_words(self, stream=None, dtype=np.int64):
        """The int forms' accumulated root tensor: 64-bit words (the sums
        modulo 2^64, or residues modulo the program's modulus) read as
        ``dtype`` (``np.int64`` or ``np.uint64``)."""
        n = 1 << int(self.info.root_rank)
        out = np.zeros(n, dtype=np.uint64)
        check(lib().togb_program_result_u64(self._h, _stream_handle(stream),
                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n))
        return out.view(dtype).reshape((2,) * int(self.info.root_rank))

    def partial(self, stream=None):
        """This program's accumulated result as a sharding partial: the
        compensated sum (rounded once) and a zero compensation."""
        out = self.result(stream).reshape(-1)
        return out, np.zeros_like(out)

    def set_timing(self, enable=True):
        check(lib().togb_program_set_timing(self._h, 1 if enable else 0))

    def set_wait_limit(self, cycles=0):
        """Limit of every device-side wait in SM clock cycles (<= 0: the
        default, about one second).  An expired wait makes :meth:`result`
        raise ``TogbError`` with status ``ERR_TIMEOUT``."""
        check(lib().togb_program_set_wait_limit(self._h, int(cycles)))

    def join_times(self):
        n = int(self.info.num_joins)
        out = (ctypes.c_float * n)()
        check(lib().togb_program_join_times(self._h, out, n))
        return np.array(out, dtype=np.float64)

    def joins(self, mode):
        """Per join: (log2 M, log2 N, log2 K, kernel id, runs per slice) as an
        int array [joins, 5]; the last column is 0 for slice-invariant joins,
        which run once per call."""
        n = int(self.info.num_joins)
        out = np.zeros((max(n, 1), 5), dtype=np.int32)
        check(lib().togb_program_joins(self._h, int(mode), out.ctypes.data_as(_i32p), n))
        return out[:n]

    def describe(self, mode, join):
        """The library's description of join ``join`` in ``mode``: shape,
        kernel, operand layouts (as the last run in ``mode`` lowered them)."""
        buf = ctypes.create_string_buffer(8192)
        check(lib().togb_program_describe(self._h, int(mode), int(join), buf, 8192))
        return buf.value.decode()

    def launch_count(self, mode):
        """Kernel launches of one count in ``mode`` as the last run queued them."""
        out = ctypes.c_int64()
        check(lib().togb_program_launch_count(self._h, int(mode), ctypes.byref(out)))
        return int(out.value)

    def set_kernel(self, mode, join, kernel):
        """Run ``join`` with ``kernel`` (an id of ``KERNEL_NAMES``; -1 = default) in ``mode``."""
        check(lib().togb_program_set_kernel(self._h, int(mode), int(join), int(kernel)))

    def kernel_allowed(self, mode, join, kernel):
        out = ctypes.c_int32()
        check(lib().togb_program_kernel_allowed(self._h, int(mode), int(join), int(kernel), ctypes.byref(out)))
        return bool(out.value)

    def allowed_kernels(self, mode):
        """Per join, the kernel ids it may run in ``mode``."""
        return [[k for k in KERNEL_NAMES if self.kernel_allowed(mode, j, k)] for j in range(int(self.info.num_joins))]

    def close(self):
        if getattr(self, "_h", None):
            lib().togb_program_destroy(self._h)
            self._h = None
        self._workspace = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tensordot_f64(a, b, axes, out=None, stream=None):
    """``np.tensordot(a, b, axes)`` for binary-index FP64 CUDA tensors (torch)."""
    import torch

    return _tensordot(a, b, axes, out, stream, torch.float64, lib().togb_tensordot_f64)


def tensordot_i64(a, b, axes, out=None, stream=None):
    """``np.tensordot(a, b, axes)`` for binary-index int64 CUDA tensors (torch),
    sums and products modulo 2^64 as numpy computes int64 and uint64 tensors."""
    import torch

    return _tensordot(a, b, axes, out, stream, torch.int64, lib().togb_tensordot_i64)


def _tensordot(a, b, axes, out, stream, dtype, entry):
    import torch

    axes_a, axes_b = [list(x) for x in axes]
    if len(axes_a) != len(axes_b):
        raise ValueError("shape-mismatch for sum")
    for t in (a, b):
        if t.dtype != dtype or not t.is_cuda:
            raise TypeError("tensordot takes %s CUDA tensors" % dtype)
        if any(d != 2 for d in t.shape):
            raise ValueError("only binary (dimension-2) indices are supported")
    ra, rb = a.dim(), b.dim()
    axes_a = [x % ra if ra else x for x in axes_a]
    axes_b = [x % rb if rb else x for x in axes_b]
    a = a.contiguous()
    b = b.contiguous()
    rank = ra + rb - 2 * len(axes_a)
    if out is None:
        out = torch.empty((2,) * rank, dtype=dtype, device=a.device)
    aa = np.array(axes_a or [0], dtype=np.int32)
    bb = np.array(axes_b or [0], dtype=np.int32)
    check(entry(ctypes.c_void_p(a.data_ptr()), ra, ctypes.c_void_p(b.data_ptr()), rb,
                len(axes_a), aa.ctypes.data_as(_i32p), bb.ctypes.data_as(_i32p),
                ctypes.c_void_p(out.data_ptr()), _stream_handle(stream)))
    return out


def probe_peak(kind, stream=None):
    """Measured FMA throughput in FLOP/s: kind 0 = FP64, 1 = FP32."""
    v = ctypes.c_double()
    check(lib().togb_probe_peak(int(kind), _stream_handle(stream), ctypes.byref(v)))
    return v.value


def contract_static_f64(program: Program, leaf_values, out, stream=None):
    """FP64 contraction through ``togb_contract_static_f64``: no device memory
    is allocated by the library.  ``leaf_values`` is a float64 CUDA tensor with
    the concatenated leaf parents (``DeviceProgram``'s layout) and ``out`` a
    float64 CUDA tensor of ``2**root_rank`` entries; both belong to the caller.
    Calls that overlap on the GPU share one scratch array and must not run
    concurrently.

    Both tensors are checked before anything is queued (``ValueError``): the
    library receives raw addresses and sizes them from the program alone, so a
    short, strided, mistyped or foreign-device buffer would be read or written
    out of bounds on the device."""
    import torch

    n_values = sum(1 << l.rank for l in program.leaves)
    n_out = 1 << program_root_rank(program)
    for name, t, want in (("leaf_values", leaf_values, None), ("out", out, n_out)):
        if not isinstance(t, torch.Tensor) or t.dtype != torch.float64:
            raise ValueError("%s must be a float64 torch tensor" % name)
        if not t.is_contiguous():
            raise ValueError("%s must be contiguous" % name)
        if want is not None and t.numel() != want:
            raise ValueError("%s holds %d entries; the root tensor has %d" % (name, t.numel(), want))
    if leaf_values.numel() < n_values:
        raise ValueError("leaf_values holds %d entries; the program's leaves need %d"
                         % (leaf_values.numel(), n_values))
    if not (leaf_values.is_cuda and out.is_cuda):
        raise ValueError("leaf_values and out must be CUDA tensors")
    if leaf_values.device != out.device:
        raise ValueError("leaf_values (%s) and out (%s) are on different devices" % (leaf_values.device, out.device))
    with torch.cuda.device(out.device):
        return _contract_static_f64(program, leaf_values, out, stream)


def program_root_rank(program: Program):
    """Rank of the final tensor over unsliced edges: the edges of the root
    that the post-order walk leaves uncontracted (0 for a count)."""
    from .program import join_edges

    sliced = {e for g in program.slice_groups for e in g}
    stack = []
    for t in program.postorder:
        if t >= 0:
            stack.append([e for e in program.leaves[t].axes if e not in sliced])
        else:
            r = stack.pop()
            l = stack.pop()
            stack.append(join_edges(l, r)[2])
    return len(stack[0])


def _contract_static_f64(program, leaf_values, out, stream):
    leaves = program.leaves
    ranks = np.array([l.rank for l in leaves], dtype=np.int32)
    axes = np.array([a for l in leaves for a in l.axes] or [0], dtype=np.int32)
    tokens = np.array(program.postorder, dtype=np.int32)
    gsize = np.array([len(g) for g in program.slice_groups] or [0], dtype=np.int32)
    gedges = np.array([e for g in program.slice_groups for e in g] or [0], dtype=np.int32)
    desc = ProgramDesc(len(leaves), ranks.ctypes.data_as(_i32p), axes.ctypes.data_as(_i32p), None,
                       len(tokens), tokens.ctypes.data_as(_i32p), len(program.slice_groups),
                       gsize.ctypes.data_as(_i32p), gedges.ctypes.data_as(_i32p))
    check(lib().togb_contract_static_f64(ctypes.byref(desc), ctypes.c_void_p(leaf_values.data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()), _stream_handle(stream)))
    return out
