"""The plugin returns to Python between bounded calls, so the reference's
SIGALRM timeout can interrupt a count (no GPU needed).

``util.TimeoutTimer`` (``src/util/util.py:13-122``) arms ``signal.alarm`` and
raises ``TimeoutError`` from the handler (``util.py:32-39``); Python runs the
handler only when the main thread is back in the interpreter.  The device
program here is a stand-in whose calls take wall time, so the test checks the
host loop alone: calls are sized to ``max_call_seconds`` from the measured time
of the previous call, the wait returns to the interpreter, and the timeout
leaves the remaining slices unqueued.
"""
import signal
import time

import numpy as np
import pytest

from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Leaf, Program


class FakeInfo:
    flops_per_slice = 1e9
    root_rank = 0


class FakeDeviceProgram:
    """Each slice costs ``SLICE_SECONDS`` of 'device' time, spent in the wait."""

    SLICE_SECONDS = 0.002
    calls = []

    def __init__(self, program, device=0):
        self.info = FakeInfo()
        self.pending = 0.0
        self.total = 0.0

    def reset(self, stream=None):
        self.total = 0.0

    def allocate_workspace(self, mode, slices, max_fraction=0.5):
        return None

    def run(self, mode, begin=0, end=None, workspace=None, stream=None):
        FakeDeviceProgram.calls.append((begin, end))
        self.pending += (end - begin) * self.SLICE_SECONDS
        self.total += end - begin

    def result(self, stream=None):
        return np.array(self.total)


def program(groups):
    leaves = [Leaf([i], "var", w_neg=0.5, w_pos=0.5) for i in range(groups)]
    tokens = [0] + [t for i in range(1, groups) for t in (i, -1)]
    return Program(leaves, tokens, [[i] for i in range(groups)])


@pytest.fixture
def fake(monkeypatch):
    FakeDeviceProgram.calls = []
    monkeypatch.setattr(runtime, "DeviceProgram", FakeDeviceProgram)
    monkeypatch.setattr(api.GB300API, "_stream", lambda self: None)

    def wait(stream):
        dp = api_under_test.last_program
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < dp.pending:
            time.sleep(1e-4)  # back in the interpreter between polls
        dp.pending = 0.0

    monkeypatch.setattr(api.GB300API, "_wait", staticmethod(wait))


api_under_test = None


def test_calls_are_sized_to_the_time_target(fake):
    global api_under_test
    api_under_test = api.GB300SplitAPI()
    api_under_test.max_call_seconds = 0.02
    value = api_under_test.contract_program(program(8))  # 256 slices of 2 ms
    assert value == 256
    calls = FakeDeviceProgram.calls
    assert calls[0][0] == 0 and calls[-1][1] == 256
    assert all(a[1] == b[0] for a, b in zip(calls, calls[1:]))
    # after the first call every call holds about 0.02 s / 2 ms = 10 slices
    assert all(5 <= e - s <= 20 for s, e in calls[1:-1])


def test_sigalrm_timeout_interrupts_the_count(fake):
    global api_under_test
    api_under_test = api.GB300SplitAPI()
    api_under_test.max_call_seconds = 0.02

    def handler(signum, frame):
        raise TimeoutError()

    old = signal.signal(signal.SIGALRM, handler)
    signal.setitimer(signal.ITIMER_REAL, 0.1)
    try:
        t0 = time.perf_counter()
        with pytest.raises(TimeoutError):
            api_under_test.contract_program(program(10))  # 1024 slices of 2 ms: about 2 s
        elapsed = time.perf_counter() - t0
    finally:
        signal.setitimer(signal.ITIMER_REAL, 0)
        signal.signal(signal.SIGALRM, old)
    assert elapsed < 0.5
    queued = FakeDeviceProgram.calls[-1][1]
    assert queued < 1024  # the rest of the count was never queued
