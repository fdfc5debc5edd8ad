"""Failure detection of the persistent kernel's grid barrier, on the GPU,
without a fault: the wait is made to run out and the error status is read.

ifx_set_barrier_fault starts the next launch's arrival counter one short, as if
one of its blocks had been lost, and gives every barrier a short poll limit.
Every block then gives up at the first barrier and returns; the step reports
IFX_ERR_CUDA, the handle refuses further steps with IFX_ERR_STATE, and the
device stays usable: a new handle on the same device steps and agrees bit for
bit with a handle that never saw the fault.
"""
import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu


def spec():
    return cases.external(64, 48, 12.0, 8.0, 4.0, 4.0, 0.5, 0.5, 0.0, 100.0, 1e-2, capi.PREC_FP64, ratio=4.0,
                          width=1.0)


def test_grid_barrier_wait_runs_out_and_is_reported():
    lib = ifx.lib()
    s = ifx.Solver.create(*spec())
    s.set_exec_mode(ifx.EXEC_PERSISTENT)
    s.step(1)
    # about 2000 polls of ~100 ns: the launch ends within a millisecond
    assert lib.ifx_set_barrier_fault(s._h, 2000, 1) == capi.IFX_OK
    with pytest.raises(ifx.IFXError) as e:
        s.step(1)
    assert e.value.status == capi.IFX_ERR_CUDA and "grid barrier timed out" in str(e.value)
    with pytest.raises(ifx.IFXError) as e:
        s.step(1)
    assert e.value.status == capi.IFX_ERR_STATE
    s.close()
    # the device is still usable
    a = ifx.Solver.create(*spec())
    a.set_exec_mode(ifx.EXEC_PERSISTENT)
    a.step(2)
    b = ifx.Solver.create(*spec())
    b.set_exec_mode(ifx.EXEC_GRAPH)
    b.step(2)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
        assert np.array_equal(a.get(f), b.get(f)), f


def test_short_spin_limit_alone_does_not_fail_a_step():
    # a limit without a withheld arrival only bounds the wait: every barrier
    # completes long before 10^5 polls, and the step equals an untouched run
    lib = ifx.lib()
    a = ifx.Solver.create(*spec())
    a.set_exec_mode(ifx.EXEC_PERSISTENT)
    assert lib.ifx_set_barrier_fault(a._h, 100000, 0) == capi.IFX_OK
    a.step(1)
    b = ifx.Solver.create(*spec())
    b.set_exec_mode(ifx.EXEC_PERSISTENT)
    b.step(1)
    assert np.array_equal(a.get(capi.FIELD_U), b.get(capi.FIELD_U))
