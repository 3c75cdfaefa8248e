"""Timeouts on the device path.

* A device-side wait that runs out.  The fused slice-invariant list
  (``k_once_list``) waits, bounded, for producer tiles that other CTAs of the
  same launch publish.  With the program's wait limit set to one clock cycle a
  consumer tile that finds its producer unfinished gives up at once, sets the
  program's error word and its CTA returns; ``togb_program_result`` must then
  report ``TOGB_ERR_TIMEOUT``, and the next run with the default limit must
  give the same bits as a run before the expiry.  The plain FP64 form is used,
  so no tensor-core kernel runs with the shortened limit.
* The reference's SIGALRM timeout (``util.py:32-39`` raises ``TimeoutError``
  from the handler) interrupting a count: the plugin queues calls of bounded
  device time and polls for them from Python.
"""
import gzip
import json
import os
import signal
import time

import numpy as np
import pytest

from conftest import ROOT
from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu


def workload():
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc220_s10.json.gz"), "rt") as f:
        doc = json.load(f)
    return Program.from_dict(doc["program"]), doc["reference"]["float64"]


def test_expired_wait_reports_timeout_then_recovers(cuda):
    prog, _ = workload()
    dp = runtime.DeviceProgram(prog)
    mode, slices = runtime.MODE_F64, 8

    def count():
        dp.reset()
        dp.run(mode, 0, slices)
        return dp.result().copy()

    before = count()
    dp.set_wait_limit(1)
    statuses = []
    for _ in range(5):  # a consumer tile almost surely finds a producer unfinished
        try:
            count()
            statuses.append(runtime.OK)
        except runtime.TogbError as exc:
            statuses.append(exc.status)
            assert "wait ran out" in str(exc)
            break
    assert runtime.ERR_TIMEOUT in statuses
    dp.set_wait_limit(0)  # the default again
    after = count()
    assert np.array_equal(before, after)
    dp.close()


def test_sigalrm_interrupts_a_device_count(cuda):
    import torch

    prog, ref = workload()
    plain = api.GB300API()
    plain.max_call_seconds = 0.05  # the plain form's count takes about a second

    def handler(signum, frame):
        raise TimeoutError()

    old = signal.signal(signal.SIGALRM, handler)
    try:
        plain.contract_program(prog, num_slice_limit=16)  # warm: library, context, workspace
        signal.setitimer(signal.ITIMER_REAL, 0.25)
        t0 = time.perf_counter()
        with pytest.raises(TimeoutError):
            plain.contract_program(prog)
        elapsed = time.perf_counter() - t0
    finally:
        signal.setitimer(signal.ITIMER_REAL, 0)
        signal.signal(signal.SIGALRM, old)
    assert elapsed < 0.6
    torch.cuda.synchronize()
    # the device is usable and the count is intact afterwards
    got = float(api.GB300SplitAPI().contract_program(prog))
    assert abs(got - ref) <= 1e-6 * abs(ref)
