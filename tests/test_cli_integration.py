"""The plugin inside the reference's own CLI (tensororder.py run): registration
makes --tensor_library gb300 / gb300-split resolve, and the Execution stage
hands the plugin the planned network.  Needs the reference checkout and the
oracle build (python oracle/build_ref.py); skipped elsewhere.  The device call
is replaced by the oracle here -- this test checks the wiring, not the compute
(the GPU parity tests check the compute)."""
import io
import os
import sys

import numpy as np
import pytest

from oracle import refload

pytestmark = pytest.mark.skipif(not refload.available(), reason="reference checkout / oracle build absent")


@pytest.mark.parametrize("library,entry,mode", [("gb300", "float64", 0), ("gb300-split", "float64", 1),
                                                ("gb300", "float32", 1), ("gb300", "int", 2),
                                                ("gb300-split", "uint", 2), ("gb300", "bigint", "exact")])
def test_cli_selects_plugin(library, entry, mode, monkeypatch, capsys):
    refload.load()
    from oracle import contract
    from tensororder_gb300 import api, launcher

    calls = []

    def stub(self, prog, limit):
        calls.append((prog.num_joins, prog.num_slices, "exact" if self._bigint else self._mode))
        if self._bigint:
            return np.asarray(int(contract.contract_sliced(prog, limit, dtype=np.int64)), dtype=object)
        dtype = self._word_type if self._mode == 2 else np.float64
        return np.asarray(contract.contract_sliced(prog, limit, dtype=dtype))

    monkeypatch.setattr(api.GB300API, "_run", stub)
    monkeypatch.setattr(api, "_OOM", api._OOM)  # register() rebinds it; restore afterwards
    cnf = os.path.join(refload.reference_src(), "..", "benchmarks", "cubic_vertex_cover", "cubic_vc_50_0.cnf")
    monkeypatch.setattr(sys, "stdin", io.StringIO(open(cnf).read()))
    monkeypatch.chdir(refload.REF_OUT)
    with pytest.raises(SystemExit) as exc:
        launcher.main(["--reference-src", refload.reference_src(), "tensororder", "--planner", "line-Flow",
                       "--weights", "unweighted", "--tensor_library", library, "--timeout", "3",
                       "--minimum_slice", "2", "--entry_type", entry])
    assert exc.value.code == 0
    out = capsys.readouterr().out
    assert "Count: 2802717837" in out
    assert len(calls) == 1 and calls[0][1] == 4 and calls[0][2] == mode


@pytest.mark.gpu
@pytest.mark.parametrize("library", ["gb300", "gb300-split"])
def test_cli_counts_on_the_device(library, monkeypatch, capsys, cuda):
    """The same CLI run with the real kernels: the count must come out of
    libtogb.  Needs both the reference checkout and a GPU in one place."""
    refload.load()
    from tensororder_gb300 import api, launcher

    runs = []
    real = api.GB300API._run

    def spy(self, prog, limit):
        out = real(self, prog, limit)
        runs.append(self.last_program is not None)
        return out

    monkeypatch.setattr(api.GB300API, "_run", spy)
    monkeypatch.setattr(api, "_OOM", api._OOM)
    cnf = os.path.join(refload.reference_src(), "..", "benchmarks", "cubic_vertex_cover", "cubic_vc_50_0.cnf")
    monkeypatch.setattr(sys, "stdin", io.StringIO(open(cnf).read()))
    monkeypatch.chdir(refload.REF_OUT)
    with pytest.raises(SystemExit) as exc:
        launcher.main(["--reference-src", refload.reference_src(), "tensororder", "--planner", "line-Flow",
                       "--weights", "unweighted", "--tensor_library", library, "--timeout", "3",
                       "--minimum_slice", "2"])
    assert exc.value.code == 0
    out = capsys.readouterr().out
    assert ("Count: 2802717837" in out) if library == "gb300" else ("Count: 2802717" in out)
    assert runs == [True]
