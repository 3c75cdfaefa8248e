"""Every kernel a join may run gives the same count: each join of a few plans
is switched, one kernel id at a time, to every kernel the library allows for
it (togb_program_set_kernel), and the count must stay within the form's
tolerance of the reference's count (plain 1e-12, split 1e-6)."""
import pytest

from conftest import load_golden
from tensororder_gb300 import runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["wvc120", "vc60_s4", "r3cnf20_factor", "wvc40_early"])
@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)])
@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
def test_count_is_independent_of_kernel_choice(name, mode, tol, kernel, cuda):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    dp = runtime.DeviceProgram(prog)
    allowed = dp.allowed_kernels(mode)
    changed = 0
    for j, ks in enumerate(allowed):
        if kernel in ks:
            dp.set_kernel(mode, j, kernel)
            changed += 1
    dp.reset()
    dp.run(mode)
    got = float(dp.result())
    info = dp.joins(mode)
    dp.close()
    want = float(doc["reference"]["float64"])
    assert abs(got - want) <= tol * abs(want)
    assert sum(1 for j in range(len(allowed)) if int(info[j][3]) == kernel) >= changed


def test_disallowed_kernel_is_rejected(cuda):
    prog = Program.from_dict(load_golden("wvc120")["program"])
    dp = runtime.DeviceProgram(prog)
    allowed = dp.allowed_kernels(runtime.MODE_SPLIT)
    j = next(j for j, ks in enumerate(allowed) if 3 not in ks)
    with pytest.raises(runtime.TogbError):
        dp.set_kernel(runtime.MODE_SPLIT, j, 3)
    dp.close()
