"""The bounded device-side wait of the step kernels gives up with an error status instead of
hanging: a test hook arms an mbarrier for bytes that no copy delivers (no bulk copy is in
flight) and waits a short poll limit; the wait returns false, ABM_DIAG_TIMEOUTS counts it and
abm_vpf_status reports ABM_ERR_TIMEOUT, after which the context still runs steps normally.
(The reference has no device waits; its nearest analogue is the status-and-skip of
vf_agent.py:268, :283-284.)"""
import ctypes

import numpy as np
import pytest

from conftest import gpu_available
from _gpu_helpers import seeded_swarm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_wait_that_runs_out_reports_timeout():
    import torch
    from abm_gb300 import _lib
    lib = _lib.load()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.abm_vpf_status(1, s) == 0, "status flag set before the test"
    diag = torch.zeros(_lib.ABM_DIAG_COUNT, dtype=torch.int64, device="cuda")
    res = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    _lib.check(lib.abm_vpf_debug_wait_timeout(1024, _lib.u64ptr(diag), _lib.i32ptr(res), s))
    assert lib.abm_vpf_status(0, s) == _lib.ABM_ERR_TIMEOUT
    assert b"bounded wait" in lib.abm_last_error_string()
    assert res.item() == 0                              # the wait returned false
    assert int(diag[_lib.DIAG_TIMEOUTS].item()) == 1    # and was counted
    assert lib.abm_vpf_status(1, s) == _lib.ABM_ERR_TIMEOUT   # still set; now cleared
    assert lib.abm_vpf_status(1, s) == 0
    # a second run-out is reported again
    _lib.check(lib.abm_vpf_debug_wait_timeout(1, _lib.u64ptr(diag), _lib.i32ptr(res), s))
    assert lib.abm_vpf_status(1, s) == _lib.ABM_ERR_TIMEOUT
    assert int(diag[_lib.DIAG_TIMEOUTS].item()) == 2
    assert lib.abm_vpf_debug_wait_timeout(0, None, _lib.i32ptr(res), s) == _lib.ABM_ERR_INVALID_ARG


def test_context_usable_after_a_timeout_and_tiled_steps_report_ok():
    """After a wait ran out, the tiled (TMA-staged) step still runs on the same context, gives
    the same results as the L1 form and leaves the status clean."""
    import torch
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    lib = _lib.load()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    res = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(lib.abm_vpf_debug_wait_timeout(64, None, _lib.i32ptr(res), s))
    assert lib.abm_vpf_status(1, s) == _lib.ABM_ERR_TIMEOUT
    st = seeded_swarm(21, 3000, 3000.0, 3000.0, R=5.0)
    vp = VFParams(width=3000.0, height=3000.0, rv=1200, radius=5.0)
    outs = []
    try:
        for mode, warps, tile in ((2, 8, 1024), (1, 8, 8192)):
            _lib.check(lib.abm_vpf_set_step_mode(mode, 1))
            _lib.check(lib.abm_vpf_set_step_config(warps, tile))
            sw = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
            sw.step(want_vpf=True, want_terms=True)
            sw.check_status()
            assert sw.diagnostics()["timeouts"] == 0
            outs.append((sw.vpf_numpy(), sw.terms.cpu().numpy()))
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
        lib.abm_vpf_set_step_config(8, 8192)
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
