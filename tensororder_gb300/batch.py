"""Uneven batches: many instances, each with its own plan and slice count,
contracted by one CUDA graph per step, with per-join kernels picked by an
autotuner.

* :class:`Autotuner` times every kernel a join may run (timing mode, CUDA
  events per launch; :func:`learned.record_timings`) on a sample of the
  batch and keeps, per join shape (log2 M, N, K, which operands are leaves,
  slices per launch), the fastest kernel.  Joins of shapes it has not timed
  keep the library's default kernel.
* :class:`BatchExecutor` creates every instance's device program and
  workspace, applies the tuned kernels, and builds one ``togb_batch``: a CUDA
  graph in which each instance's whole count runs on one of ``nstreams``
  internal streams.  :meth:`BatchExecutor.run` replays it (one step = every
  instance's count); :meth:`BatchExecutor.counts` reads the counts back.

The reference contracts instances one at a time, each through
``execution.run`` (``execution.py:122-152``).
"""
from __future__ import annotations

import ctypes
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import costmodel, learned, runtime
from .program import Program

ShapeKey = Tuple[int, int, int, int, bool, bool, int]


def shape_key(j: costmodel.JoinShape, slices: int, mode: int) -> ShapeKey:
    return (mode, j.lm, j.ln, j.lk, j.left_leaf, j.right_leaf, int(round(math.log2(max(1, slices)))))


class Autotuner:
    """Fastest measured kernel per join shape."""

    def __init__(self, mode: int):
        self.mode = mode
        self.best: Dict[ShapeKey, Tuple[int, float]] = {}
        self.rows: List[learned.TimingRow] = []

    def tune(self, programs: Sequence[Program], repeats: int = 2, device: int = 0) -> int:
        """Time the joins of ``programs``; returns how many shapes are known."""
        for prog in programs:
            rows = learned.record_timings(prog, self.mode, repeats=repeats, device=device)
            self.rows.extend(rows)
            for r in rows:
                f = r.features
                kernel = int(np.argmax(f[12:16]))
                key = (self.mode, int(f[0]), int(f[1]), int(f[2]), bool(f[9]), bool(f[10]), int(round(f[6])))
                if key not in self.best or r.ms < self.best[key][1]:
                    self.best[key] = (kernel, r.ms)
        return len(self.best)

    def kernels_for(self, program: Program, slices_per_launch: int) -> List[int]:
        out = []
        for j in costmodel.join_table(program):
            nb = slices_per_launch if j.per_slice else 1
            hit = self.best.get(shape_key(j, nb, self.mode))
            out.append(hit[0] if hit else -1)
        return out


class BatchExecutor:
    """All instances of a batch as one CUDA graph (see module doc)."""

    def __init__(self, programs: Sequence[Program], mode: int, device: int = 0, nstreams: int = 16,
                 tuner: Optional[Autotuner] = None, max_fraction: float = 0.5):
        import torch

        self.mode = mode
        self.device = device
        self.programs = list(programs)
        self.dps = [runtime.DeviceProgram(p, device) for p in self.programs]
        free, _ = torch.cuda.mem_get_info(device)
        budget = free * max_fraction
        need = sum(dp.workspace_bytes(mode, dp.num_slices) for dp in self.dps)
        scale = min(1.0, budget / max(1.0, need))
        self.ws = []
        for dp in self.dps:
            per = int(dp.info.workspace_per_slice[mode])
            fixed = int(dp.info.workspace_fixed[mode])
            slices = max(1, min(dp.num_slices, int(dp.num_slices * scale)))
            self.ws.append(torch.empty(per * slices + fixed, dtype=torch.uint8, device=torch.device("cuda", device)))
        self.kernels_applied = 0
        if tuner is not None:
            for prog, dp, w in zip(self.programs, self.dps, self.ws):
                B = min(dp.num_slices, (w.numel() - int(dp.info.workspace_fixed[mode])) //
                        max(1, int(dp.info.workspace_per_slice[mode])))
                for j, k in enumerate(tuner.kernels_for(prog, B)):
                    if k >= 0 and dp.kernel_allowed(mode, j, k):
                        dp.set_kernel(mode, j, k)
                        self.kernels_applied += 1
        n = len(self.dps)
        handles = (ctypes.c_void_p * n)(*[dp._h.value for dp in self.dps])
        wsp = (ctypes.c_void_p * n)(*[w.data_ptr() for w in self.ws])
        wsb = (ctypes.c_size_t * n)(*[w.numel() for w in self.ws])
        out = ctypes.c_void_p()
        runtime.check(runtime.lib().togb_batch_create(handles, n, int(mode), wsp, wsb, int(nstreams), ctypes.byref(out)))
        self._h = out

    @property
    def h2d_bytes(self) -> int:
        return int(sum(dp.h2d_bytes for dp in self.dps))

    def run(self, stream=None):
        runtime.check(runtime.lib().togb_batch_run(self._h, runtime._stream_handle(stream)))

    def counts(self, stream=None) -> np.ndarray:
        out = np.zeros(len(self.dps), dtype=np.float64)
        runtime.check(runtime.lib().togb_batch_results(self._h, runtime._stream_handle(stream),
                                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                       len(self.dps)))
        return out

    def work(self) -> Dict[str, float]:
        flops = sum(costmodel.executed_cost(p)["flops"] for p in self.programs)
        return {"instances": len(self.programs), "slices": sum(p.num_slices for p in self.programs),
                "executed_flops": flops}

    def close(self):
        if getattr(self, "_h", None):
            runtime.lib().togb_batch_destroy(self._h)
            self._h = None
        for dp in self.dps:
            dp.close()
        self.ws = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
