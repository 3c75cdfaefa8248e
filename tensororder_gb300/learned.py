"""The learned cost model: a small MLP that predicts the device time of every
join launch from its shape, kernel and slice width, trained on timings the
backend records itself, and the selector that uses it.

* :class:`MLP` -- the network (F -> 128 -> 128 -> 1, FP32) with its forward,
  backward and Adam update run by this package's own CUDA kernels
  (``csrc/togb_mlp.cu``); torch only provides the device buffers.
* :func:`join_features` -- the per-launch feature vector: log2 extents, output
  and operand ranks, slices in the launch, FLOPs and bytes of the launch,
  which operands are leaves, the kernel and the form.
* :func:`record_timings` -- runs a program with every kernel a join may use
  (timing mode: CUDA events around each launch) and returns one
  ``(features, ms)`` row per join launch.
* :class:`Selector` -- picks the slice set (among
  :func:`costmodel.slice_candidates`) and the kernel of every join that the
  model predicts to be fastest; without a trained model, or when a prediction
  is not finite, it falls back to the plain FLOP/memory model
  (:func:`costmodel.flop_model_seconds`) and the default kernels.  Any choice
  gives the same count -- slice sets partition the same sum and every kernel
  computes the same contraction -- so the model can change only the speed.

The reference has no learned component; its planner ranks plans by the
FLOP/memory estimate of ``contraction_methods/contraction_tree.pyx:382-496``.
"""
from __future__ import annotations

import ctypes
import json
import math
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import costmodel, runtime
from .program import Program

KERNELS = (0, 1, 2, 3)
NUM_FEATURES = 17
_fp = ctypes.POINTER(ctypes.c_float)


def join_features(j: costmodel.JoinShape, kernel: int, slices: int, mode: int) -> np.ndarray:
    """Feature vector of one launch of join ``j`` over ``slices`` slices."""
    f = np.zeros(NUM_FEATURES, dtype=np.float32)
    lb = math.log2(max(1, slices))
    f[0:3] = (j.lm, j.ln, j.lk)
    f[3] = j.lm + j.ln
    f[4] = j.lm + j.lk
    f[5] = j.ln + j.lk
    f[6] = lb
    f[7] = math.log2(j.flops) + lb
    f[8] = math.log2(j.bytes(4 if mode == runtime.MODE_SPLIT else 8)) + lb
    f[9] = float(j.left_leaf)
    f[10] = float(j.right_leaf)
    f[11] = float(mode == runtime.MODE_SPLIT)
    f[12 + kernel] = 1.0
    f[16] = min(j.lm, j.ln)
    return f


def _lib():
    L = runtime.lib()
    if not getattr(L, "_mlp_bound", False):
        c_void = ctypes.c_void_p
        L.togb_mlp_param_count.restype = ctypes.c_int64
        L.togb_mlp_param_count.argtypes = [ctypes.c_int, ctypes.c_int]
        L.togb_mlp_scratch_floats.restype = ctypes.c_int64
        L.togb_mlp_scratch_floats.argtypes = [ctypes.c_int, ctypes.c_int]
        L.togb_mlp_forward.restype = ctypes.c_int
        L.togb_mlp_forward.argtypes = [c_void, ctypes.c_int, ctypes.c_int, c_void, ctypes.c_int, c_void, c_void, c_void]
        L.togb_mlp_loss_grad.restype = ctypes.c_int
        L.togb_mlp_loss_grad.argtypes = [c_void, ctypes.c_int, ctypes.c_int, c_void, c_void, ctypes.c_int, c_void,
                                         c_void, c_void, c_void]
        L.togb_mlp_adam.restype = ctypes.c_int
        L.togb_mlp_adam.argtypes = [c_void, c_void, c_void, c_void, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_int32, c_void]
        L._mlp_bound = True
    return L


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class MLP:
    """F -> H -> H -> 1 network whose parameters live on the device."""

    def __init__(self, F: int = NUM_FEATURES, H: int = 128, seed: int = 0, device: int = 0):
        import torch

        self.F, self.H, self.device = F, H, device
        self.n = int(_lib().togb_mlp_param_count(F, H))
        rng = np.random.default_rng(seed)
        p = np.concatenate([
            rng.normal(0, math.sqrt(2.0 / F), F * H), np.zeros(H),
            rng.normal(0, math.sqrt(2.0 / H), H * H), np.zeros(H),
            rng.normal(0, math.sqrt(1.0 / H), H), np.zeros(1)]).astype(np.float32)
        dev = torch.device("cuda", device)
        self.params = torch.from_numpy(p).to(dev)
        self.grads = torch.zeros_like(self.params)
        self._m = torch.zeros_like(self.params)
        self._v = torch.zeros_like(self.params)
        self._loss = torch.zeros(1, dtype=torch.float32, device=dev)
        self.step = 0

    def _scratch(self, B):
        import torch

        return torch.empty(int(_lib().togb_mlp_scratch_floats(B, self.H)), dtype=torch.float32,
                           device=self.params.device)

    def _dev(self, a):
        import torch

        return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=self.params.device)

    def forward(self, x) -> np.ndarray:
        import torch

        xd = self._dev(x)
        B = xd.shape[0]
        y = torch.empty(B, dtype=torch.float32, device=self.params.device)
        st = torch.cuda.current_stream(self.device).cuda_stream
        runtime.check(_lib().togb_mlp_forward(_ptr(self.params), self.F, self.H, _ptr(xd), B, _ptr(y),
                                              _ptr(self._scratch(B)), ctypes.c_void_p(st)))
        return y.cpu().numpy()

    def loss_grad(self, x, target) -> Tuple[float, np.ndarray]:
        import torch

        xd, td = self._dev(x), self._dev(target)
        B = xd.shape[0]
        st = torch.cuda.current_stream(self.device).cuda_stream
        runtime.check(_lib().togb_mlp_loss_grad(_ptr(self.params), self.F, self.H, _ptr(xd), _ptr(td), B,
                                                _ptr(self.grads), _ptr(self._loss), _ptr(self._scratch(B)),
                                                ctypes.c_void_p(st)))
        return float(self._loss.item()), self.grads.cpu().numpy()

    def train(self, x, target, epochs=2000, lr=2e-3, batch=None, seed=0) -> List[float]:
        """Adam on the mean squared error; full batches unless ``batch``."""
        import torch

        xd, td = self._dev(x), self._dev(target)
        N = xd.shape[0]
        st = torch.cuda.current_stream(self.device).cuda_stream
        rng = np.random.default_rng(seed)
        B = N if batch is None else min(batch, N)
        scratch = self._scratch(B)
        losses = []
        for ep in range(epochs):
            if B < N:
                idx = torch.as_tensor(rng.choice(N, B, replace=False), device=xd.device)
                xb, tb = xd[idx].contiguous(), td[idx].contiguous()
            else:
                xb, tb = xd, td
            runtime.check(_lib().togb_mlp_loss_grad(_ptr(self.params), self.F, self.H, _ptr(xb), _ptr(tb), B,
                                                    _ptr(self.grads), _ptr(self._loss), _ptr(scratch),
                                                    ctypes.c_void_p(st)))
            self.step += 1
            runtime.check(_lib().togb_mlp_adam(_ptr(self.params), _ptr(self.grads), _ptr(self._m), _ptr(self._v),
                                               self.n, lr, 0.9, 0.999, 1e-8, self.step, ctypes.c_void_p(st)))
            if ep % 50 == 0 or ep == epochs - 1:
                losses.append(float(self._loss.item()))
        return losses

    def state(self) -> Dict:
        return {"F": self.F, "H": self.H, "params": self.params.cpu().numpy().tolist()}

    def load_state(self, d):
        import torch

        if d["F"] != self.F or d["H"] != self.H:
            raise ValueError("network shape mismatch")
        self.params = torch.tensor(d["params"], dtype=torch.float32, device=self.params.device)


@dataclass
class TimingRow:
    features: np.ndarray
    ms: float


def record_timings(program: Program, mode: int, kernels: Sequence[int] = KERNELS, repeats: int = 2,
                   device: int = 0, max_slices: Optional[int] = None) -> List[TimingRow]:
    """Per-launch device times of every join of ``program`` under each kernel
    it may run: one timed pass per kernel id (joins that cannot run it keep
    their default kernel), the first ``max_slices`` slices in one chunk.  Id
    -1 is a pass with every join on its default kernel, recorded under the id
    of that kernel."""
    import torch

    dp = runtime.DeviceProgram(program, device)
    S = dp.num_slices if max_slices is None else min(dp.num_slices, max_slices)
    ws = dp.allocate_workspace(mode, S, max_fraction=0.5)
    B = min(S, (ws.numel() - int(dp.info.workspace_fixed[mode])) // max(1, int(dp.info.workspace_per_slice[mode])))
    table = costmodel.join_table(program)
    allowed = dp.allowed_kernels(mode)
    defaults = [int(x) for x in dp.joins(mode)[:, 3]]
    rows: List[TimingRow] = []
    dp.set_timing(True)
    for k in kernels:
        for j, ks in enumerate(allowed):
            dp.set_kernel(mode, j, k if k in ks else -1)
        for _ in range(repeats):  # the last pass's times are kept
            dp.reset()
            dp.run(mode, 0, B, workspace=ws)
        torch.cuda.synchronize(device)
        t = dp.join_times()
        for j, js in enumerate(table):
            if k < 0 or k in allowed[j]:  # this join ran kernel k (its default for -1) in this pass
                kj = defaults[j] if k < 0 else k
                rows.append(TimingRow(join_features(js, kj, B if js.per_slice else 1, mode), float(t[j])))
    for j in range(len(allowed)):
        dp.set_kernel(mode, j, -1)
    dp.close()
    return rows


class LearnedCostModel:
    """MLP over normalised join features predicting log(ms per launch)."""

    def __init__(self, device: int = 0, seed: int = 0):
        self.net = MLP(NUM_FEATURES, 128, seed=seed, device=device)
        self.mu = np.zeros(NUM_FEATURES, dtype=np.float32)
        self.sigma = np.ones(NUM_FEATURES, dtype=np.float32)
        self.trained = False

    def fit(self, rows: Sequence[TimingRow], epochs=3000, lr=2e-3, batch=None) -> List[float]:
        X = np.stack([r.features for r in rows]).astype(np.float32)
        y = np.log(np.maximum([r.ms for r in rows], 1e-4)).astype(np.float32)
        self.mu = X.mean(0)
        self.sigma = np.where(X.std(0) > 1e-6, X.std(0), 1.0).astype(np.float32)
        losses = self.net.train((X - self.mu) / self.sigma, y, epochs=epochs, lr=lr, batch=batch)
        self.trained = True
        return losses

    def predict_ms(self, feats: np.ndarray) -> np.ndarray:
        X = (np.atleast_2d(feats).astype(np.float32) - self.mu) / self.sigma
        return np.exp(self.net.forward(X).astype(np.float64))

    def save(self, path):
        with open(path, "w") as f:
            json.dump({"mu": self.mu.tolist(), "sigma": self.sigma.tolist(), "net": self.net.state()}, f)

    def load(self, path):
        with open(path) as f:
            d = json.load(f)
        self.mu = np.array(d["mu"], dtype=np.float32)
        self.sigma = np.array(d["sigma"], dtype=np.float32)
        self.net.load_state(d["net"])
        self.trained = True


@dataclass
class Choice:
    program: Program
    kernels: List[int]          # per join; -1 = default
    predicted_s: float
    method: str                 # "learned" or "flop-model"


def allowed_kernels_host(j: costmodel.JoinShape, mode: int) -> List[int]:
    """The kernels ``togb_program_kernel_allowed`` accepts for a join."""
    leaf = j.left_leaf or j.right_leaf
    out = [0]
    if mode == runtime.MODE_F64 or not leaf:
        out.append(1)
    if j.lm + j.ln <= 20:
        out.append(2)
    if mode == runtime.MODE_SPLIT and not leaf and j.lm >= 5 and j.ln >= 5 and j.lk >= 2:
        out.append(3)
    return out


class Selector:
    """Chooses the slice set and kernels of a plan for one form."""

    def __init__(self, mode: int, model: Optional[LearnedCostModel] = None, flops_per_s: float = 1e14,
                 bytes_per_s: float = 5e12, max_workspace_bytes: float = 64e9,
                 kernels: Optional[Sequence[int]] = None):
        """``kernels``: the kernel ids the model was trained on (default: all);
        the learned choice for a join is made among those it may run."""
        self.mode = mode
        self.model = model
        self.kernels = None if kernels is None else set(kernels)
        self.flops_per_s = flops_per_s
        self.bytes_per_s = bytes_per_s
        self.max_ws = max_workspace_bytes

    def _chunk(self, per_slice_bytes: float, S: int) -> int:
        return int(max(1, min(S, self.max_ws // max(1.0, per_slice_bytes))))

    def predict_learned(self, program: Program, per_slice_bytes: float) -> Tuple[float, List[int]]:
        """Predicted time of one count and the kernel of every join (-1: its
        default).  Each join chooses among its default kernel and the kernels
        the model was trained on that it may run."""
        S = program.num_slices
        B = self._chunk(per_slice_bytes, S)
        chunks = (S + B - 1) // B
        hp = runtime.HostProgram(program)
        defaults = [int(x) for x in hp.joins(self.mode)[:, 3]]
        hp.close()
        total = 0.0
        kernels = []
        for j, d in zip(costmodel.join_table(program), defaults):
            ks = [d] + [k for k in allowed_kernels_host(j, self.mode)
                        if k != d and (self.kernels is None or k in self.kernels)]
            nb = B if j.per_slice else 1
            feats = np.stack([join_features(j, k, nb, self.mode) for k in ks])
            ms = self.model.predict_ms(feats)
            i = int(np.argmin(ms))
            kernels.append(-1 if i == 0 else ks[i])
            total += (chunks if j.per_slice else 1) * float(ms[i]) * 1e-3
        return total, kernels

    def choose(self, candidates: Sequence[Program], per_slice_bytes: Sequence[float]) -> Choice:
        """Best candidate by the learned model; the FLOP/memory model when the
        model is missing or predicts a non-finite time for every candidate."""
        if self.model is not None and self.model.trained:
            best = None
            for prog, wb in zip(candidates, per_slice_bytes):
                t, ks = self.predict_learned(prog, wb)
                if math.isfinite(t) and (best is None or t < best.predicted_s):
                    best = Choice(prog, ks, t, "learned")
            if best is not None:
                return best
        return self.choose_flop_model(candidates, per_slice_bytes)

    def choose_flop_model(self, candidates: Sequence[Program], per_slice_bytes: Sequence[float]) -> Choice:
        best = None
        for prog, wb in zip(candidates, per_slice_bytes):
            t = costmodel.flop_model_seconds(prog, self.flops_per_s, self.bytes_per_s,
                                             4 if self.mode == runtime.MODE_SPLIT else 8,
                                             slices_per_launch=self._chunk(wb, prog.num_slices))
            if best is None or t < best.predicted_s:
                best = Choice(prog, [-1] * prog.num_joins, t, "flop-model")
        return best


def workspace_per_slice(programs: Sequence[Program], mode: int, device: int = 0) -> List[float]:
    """Device workspace bytes per slice of each program (lowered by the library)."""
    out = []
    for p in programs:
        dp = runtime.DeviceProgram(p, device)
        out.append(float(dp.info.workspace_per_slice[mode]))
        dp.close()
    return out


def run_choice(choice: Choice, mode: int, repeats: int = 3, device: int = 0, max_fraction: float = 0.5,
               max_slices: Optional[int] = None) -> Tuple[float, float]:
    """Contract ``choice`` (its slice set and kernels); returns the count of
    the first ``max_slices`` slices (all by default) and the median device
    time of one pass over them in seconds."""
    import torch

    dp = runtime.DeviceProgram(choice.program, device)
    for j, k in enumerate(choice.kernels):
        if k >= 0:
            dp.set_kernel(mode, j, k)
    n = dp.num_slices if max_slices is None else min(dp.num_slices, max_slices)
    ws = dp.allocate_workspace(mode, n, max_fraction=max_fraction)
    stream = torch.cuda.current_stream(device)
    times = []
    for _ in range(repeats + 1):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        dp.reset(stream)
        a.record(stream)
        dp.run(mode, 0, n, workspace=ws, stream=stream)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b) * 1e-3)
    count = float(dp.result(stream).reshape(-1)[0])
    dp.close()
    return count, float(np.median(times[1:]))
