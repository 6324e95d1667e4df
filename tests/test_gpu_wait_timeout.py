"""The bounded device waits of the mixed policy's tile-staged reconstruct: when a wait for its bulk
copies runs out, the kernel marks the solver's error word and returns (no trap, no hang), the call
reports AFAR_ERR_CUDA with "the state is not valid", and the context stays usable.  The wait is
made to run out on purpose through the library's test hook, which arms the tile's first barrier for
16 bytes that are never issued and shortens the limit to 2^20 clocks (about half a millisecond)."""
import numpy as np
import pytest

from conftest import gpu_available, small_cases

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_reports_an_invalid_state_and_the_context_survives():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, CaseConfig, CudaSolver, _ffi, precompute

    m, W, Wb, st = small_cases()["mixed_riemann"]
    cfg = CaseConfig(stencilType=st)
    hf = precompute(m, cfg, W, Wb)
    s = CudaSolver(hf, cfg, policy="mixed")
    s.set_tuning(0)  # the tile-staged reconstruct, whose waits these are
    L = _ffi.lib()
    _ffi.check(L.afar_debug_wait_injection(0, 16, 1 << 20))
    try:
        with pytest.raises(AfarError) as err:
            s.run(1, dt=1e-4)
    finally:
        _ffi.check(L.afar_debug_wait_injection(0, 0, 0))
    assert err.value.status == 4  # AFAR_ERR_CUDA
    assert "timed out" in str(err.value) and "state is not valid" in str(err.value)
    # normal operation again: from the initial state, steps complete and stay finite
    s.upload_state(FD=hf.FD, cFD=hf.cFD, cFDold=hf.cFD)
    s.run(3, dt=1e-4)
    out = s.state()
    assert np.isfinite(out["cFD"]).all()
    ref = CudaSolver(hf, cfg, policy="mixed")
    ref.set_tuning(0)
    ref.run(3, dt=1e-4)
    assert np.array_equal(ref.state()["cFD"], out["cFD"])
    s.close()
    ref.close()
