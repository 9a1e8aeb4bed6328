"""The allocation-free step entry point (abm_vpf_flock_step_noalloc) against the regular one.

Some callers cannot allocate device memory (code inside a host framework that owns the device
memory pool, a process that reserved all device memory); the no-alloc entry point serves them
from a fixed file-scope scratch array.  This test calls both entry points through the C ABI on
calls in a row, with different swarm sizes and grids so each call has to replace the array's
previous contents, and checks that the results agree within the parity tolerances the other GPU
tests use (they are in fact expected to be bit-identical).  The cases cover the three pair
kernels the entry point uses: up to 16384 agents the group form without neighbour chunks (walls;
a torus whose width and height are exact in float32) and the one-block-per-agent form (a torus
of another width), above that the tiled form.  It also checks the size limits.  The file name
makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


def _run(lib, fn, state, params, n, rv, torch):
    from abm_gb300 import _lib
    dev = {k: torch.as_tensor(state[k], dtype=torch.float32, device="cuda") for k in state}
    out = {k: torch.empty_like(v) for k, v in dev.items()}
    words = (rv + 31) // 32
    bits = torch.zeros((n, words), dtype=torch.int32, device="cuda")
    terms = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    sin = _lib.AbmSwarmState(*[_lib.fptr(dev[k]) for k in ("x", "y", "theta", "v")])
    sout = _lib.AbmSwarmState(*[_lib.fptr(out[k]) for k in ("x", "y", "theta", "v")])
    status = fn(ctypes.byref(sin), ctypes.byref(sout), n, ctypes.byref(params), None,
                _lib.u32ptr(bits), _lib.dptr(terms), None,
                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(status)
    torch.cuda.synchronize()
    return ({k: v.cpu().numpy() for k, v in out.items()}, bits.cpu().numpy(),
            terms.cpu().numpy())


def _compare(a, b):
    out_a, bits_a, terms_a = a
    out_b, bits_b, terms_b = b
    assert np.array_equal(bits_a, bits_b)
    scale = np.maximum(np.abs(terms_b), 1e-6)
    assert np.all(np.abs(terms_a - terms_b) / scale <= 1e-5)
    for k in out_b:
        ulp = np.spacing(np.abs(out_b[k])).astype(np.float64)
        assert np.all(np.abs(out_a[k].astype(np.float64) - out_b[k]) <= 2 * ulp), k


def test_no_alloc_matches_regular_entry_point():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import torch
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    lib = _lib.load()
    rng = np.random.default_rng(77)
    cases = [(3000, 3600, 5.0, 5000.0, "walls"), (700, 1200, 10.0, 600.0, "infinite"),
             (500, 1200, 10.0, 600.3, "infinite"),   # not a float: the one-block form
             (20000, 1200, 3.0, 9000.0, "walls")]   # the last one: the tiled pair kernel
    for n, rv, R, W, boundary in cases:   # calls in a row, different grids and sizes
        state = {"x": rng.uniform(25, W + 25, n), "y": rng.uniform(25, W + 25, n),
                 "theta": rng.uniform(0, 2 * np.pi, n), "v": rng.uniform(0, 1, n)}
        params = VFParams(alp1=0.08, bet1=0.08, width=W, height=W, rv=rv, radius=R,
                          boundary=boundary).to_c()
        noalloc = _run(lib, lib.abm_vpf_flock_step_noalloc, state, params, n, rv, torch)
        regular = _run(lib, lib.abm_vpf_flock_step, state, params, n, rv, torch)
        _compare(noalloc, regular)


def test_no_alloc_rejects_sizes_beyond_its_maximum():
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    lib = _lib.load()
    buf = (ctypes.c_float * 8)()
    fp = ctypes.cast(buf, _lib.c_float_p)
    buf2 = (ctypes.c_float * 8)()
    fp2 = ctypes.cast(buf2, _lib.c_float_p)
    sin = _lib.AbmSwarmState(fp, fp, fp, fp)
    sout = _lib.AbmSwarmState(fp2, fp2, fp2, fp2)
    p = VFParams(rv=1200).to_c()
    r = lib.abm_vpf_flock_step_noalloc(ctypes.byref(sin), ctypes.byref(sout),
                                       _lib.ABM_NOALLOC_MAX_AGENTS + 1, ctypes.byref(p), None,
                                       None, None, None, None)
    assert r == _lib.ABM_ERR_INVALID_ARG
    assert b"no-alloc maximum" in lib.abm_last_error_string()
    p = VFParams(rv=_lib.ABM_NOALLOC_MAX_RV + 1).to_c()
    r = lib.abm_vpf_flock_step_noalloc(ctypes.byref(sin), ctypes.byref(sout), 10,
                                       ctypes.byref(p), None, None, None, None, None)
    assert r == _lib.ABM_ERR_RV
