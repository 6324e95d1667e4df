"""The serving queue (afar_server_*): requests of different meshes, end times and step counts,
admitted under a device-memory budget and run together as one batch.  Each result must be bitwise
the one the same solve reaches stepped in a batch of its own (a member's result does not depend on
the other members), and the budget must bound how many run at once."""
import numpy as np
import pytest

from conftest import gpu_available, small_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cases():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    out = {}
    for name, (m, W, Wb, st) in small_cases().items():
        if name == "corner_flow":
            continue
        cfg = CaseConfig(stencilType=st, CFL=0.2 if name.startswith("ffs_tri") else 0.3)
        out[name] = (precompute(m, cfg, W, Wb, want_rbf64=True), cfg)
    return out


def _alone(hf, cfg, policy, t_end, n_steps):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch, CudaSolver

    s = CudaSolver(hf, cfg, policy=policy)
    s.set_step_params(cfl=cfg.CFL, t_end=t_end)
    b = Batch(policy)
    b.add(s)
    if n_steps:
        b.run(n_steps)
    else:
        while s.time()[0] < t_end * (1 - 1e-12):
            b.run(10)
    b.close()
    st = s.state()
    s.close()
    return st


REQS = [("quad_riemann", 0.02, 0), ("ffs_tri", 0.0, 7), ("mixed_riemann", 0.0, 12), ("quad_riemann", 0.0, 3)]


@pytest.mark.parametrize("policy", ["mixed", "fp64"])
def test_server_results_match_alone(cases, policy):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Server

    srv = Server(policy, chunk_steps=5)
    ids = [srv.submit(*cases[n], t_end=t, n_steps=k) for n, t, k in REQS]
    for rid, (n, t, k) in zip(ids, REQS):
        FD, si, lat = srv.wait(rid, timeout=120.0)
        ref = _alone(*cases[n], policy, t, k)
        assert np.array_equal(FD, ref["FD"]), n
        assert np.array_equal(si, ref["shockIndicator"]), n
        assert lat > 0
    st = srv.stats()
    assert st["completed"] == len(REQS) and st["failed"] == 0 and st["running"] == 0
    assert st["peakRunning"] >= 2 and st["bytesInUse"] == 0
    srv.close()


def test_budget_holds_for_requests_that_fit(cases):
    """With a budget of about two of the largest requests, the device memory of the running solves
    never exceeds it (the admission model is conservative and calibrated by what was built)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver, Server

    largest = 0
    for n, _, _ in REQS:
        probe = CudaSolver(*cases[n], policy="mixed")
        largest = max(largest, probe.device_bytes())
        probe.close()
    budget = int(2.2 * largest)
    srv = Server("mixed", hbm_budget_bytes=budget, chunk_steps=4)
    ids = [srv.submit(*cases[n], t_end=t, n_steps=k) for n, t, k in REQS * 2]
    for rid in ids:
        assert srv.wait(rid, timeout=120.0) is not None
    st = srv.stats()
    assert st["completed"] == 2 * len(REQS) and st["peakBytes"] <= budget
    srv.close()


def test_budget_admits_one_at_a_time(cases):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Server

    srv = Server("mixed", hbm_budget_bytes=1, chunk_steps=4)  # every request is over budget alone
    ids = [srv.submit(*cases[n], t_end=t, n_steps=k) for n, t, k in REQS]
    for rid in ids:
        assert srv.wait(rid, timeout=120.0) is not None
    st = srv.stats()
    assert st["peakRunning"] == 1 and st["completed"] == len(REQS)
    srv.close()


def test_destroy_finishes_queued_requests(cases):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Server

    srv = Server("mixed", chunk_steps=3)
    hf, cfg = cases["quad_riemann"]
    ids = [srv.submit(hf, cfg, n_steps=6) for _ in range(3)]
    keep = srv._keep
    srv.close()  # waits for the worker, which finishes everything queued
    for rid in ids:
        FD = keep[rid][3]
        assert np.isfinite(FD).all() and (FD[:, 0] > 0).all()


def test_cancel_queued_and_running(cases):
    """afar_server_cancel: a queued request is dropped at once, a running one leaves after its
    chunk; neither writes its outputs; the rest of the queue is served as if they had not been."""
    import time

    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, Server

    srv = Server("mixed", hbm_budget_bytes=1, chunk_steps=4)  # one solve at a time: the rest queue
    long_id = srv.submit(*cases["ffs_tri"], n_steps=100000)
    queued_id = srv.submit(*cases["quad_riemann"], n_steps=10)
    ok_id = srv.submit(*cases["mixed_riemann"], n_steps=12)
    srv.cancel(queued_id)
    with pytest.raises(AfarError, match="cancel"):
        srv.wait(queued_id, timeout=60.0)
    t0 = time.time()
    while srv.stats()["running"] < 1 and time.time() - t0 < 60.0:
        time.sleep(0.01)
    srv.cancel(long_id)
    with pytest.raises(AfarError, match="cancel"):
        srv.wait(long_id, timeout=120.0)
    FD, si, lat = srv.wait(ok_id, timeout=120.0)
    assert np.array_equal(FD, _alone(*cases["mixed_riemann"], "mixed", 0.0, 12)["FD"])
    with pytest.raises(AfarError):
        srv.cancel(ok_id)  # finished
    st = srv.stats()
    assert st["cancelled"] == 2 and st["completed"] == 1 and st["failed"] == 2 and st["bytesInUse"] == 0
    srv.close()


def test_non_finite_request_fails_alone(cases):
    """A request whose state holds a NaN (injected in its host input) is failed with
    AFAR_ERR_NOT_FINITE; the solve batched beside it is unaffected (bitwise)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, Server
    from afar_cudaeuler2dmixo3rk3solver_gb300.solver import HostFields

    hf, cfg = cases["quad_riemann"]
    bad = HostFields(hf.sizes, {k: v.copy() for k, v in hf.a.items()}, hf.period)
    bad.a["FD"][7] = np.nan
    bad.a["cFD"][7] = np.nan
    srv = Server("mixed", chunk_steps=5)
    ids = [srv.submit(bad, cfg, n_steps=10), srv.submit(*cases["mixed_riemann"], n_steps=10)]
    with pytest.raises(AfarError, match="finite"):
        srv.wait(ids[0], timeout=120.0)
    FD, si, lat = srv.wait(ids[1], timeout=120.0)
    assert np.array_equal(FD, _alone(*cases["mixed_riemann"], "mixed", 0.0, 10)["FD"])
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1
    srv.close()


def test_late_arrivals_join_the_running_batch(cases):
    """Continuous batching: requests submitted after the batch has started stepping are admitted
    at the next chunk boundary while the first solve is still running, finish before it, and every
    result -- the late ones and the long one -- is bitwise its result in a batch of its own."""
    import time

    from afar_cudaeuler2dmixo3rk3solver_gb300 import Server

    long_steps = 20000  # the smooth vortex box: stays finite, keeps the batch busy for a while
    srv = Server("mixed", chunk_steps=5)
    first = srv.submit(*cases["vortex_box"], n_steps=long_steps)
    t0 = time.time()
    while srv.stats()["batchSteps"] == 0 and time.time() - t0 < 60:
        time.sleep(0.001)
    assert srv.stats()["batchSteps"] > 0, "the batch never started stepping"
    late = [("quad_riemann", 0.02, 0), ("ffs_tri", 0.0, 7), ("mixed_riemann", 0.0, 12)]
    ids = [srv.submit(*cases[n], t_end=t, n_steps=k) for n, t, k in late]
    overlap = 0
    for rid, (n, t, k) in zip(ids, late):
        FD, si, _ = srv.wait(rid, timeout=120.0)
        overlap = max(overlap, srv.stats()["peakRunning"])
        ref = _alone(*cases[n], "mixed", t, k)
        assert np.array_equal(FD, ref["FD"]), n
        assert np.array_equal(si, ref["shockIndicator"]), n
    st = srv.stats()
    assert st["completed"] == len(late) and st["running"] == 1, st  # the long solve is still stepping
    assert overlap >= 2
    FD, si, _, steps = srv.wait(first, timeout=300.0, with_steps=True)
    assert steps == long_steps
    ref = _alone(*cases["vortex_box"], "mixed", 0.0, long_steps)
    assert np.array_equal(FD, ref["FD"]) and np.array_equal(si, ref["shockIndicator"])
    srv.close()
