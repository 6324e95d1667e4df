"""The optional multi-point face flux on the GPU (afar_set_face_gauss_flux), through the C ABI:

* the 1-point rule is the face-centre flux (fp64, to 1e-12 of the flux scale; the kernels form
  densities by different divisions);
* with 3 points, the fp64 policy against the CPU oracle's restatement, stage by stage for two
  steps: every output within 1e-10 and identical switch decisions;
* the mixed policy's multi-point flux against the fp64 policy's, to FP32 rounding;
* graph-replayed steps run it, and a solver with it cannot join a batch.
"""
import numpy as np
import pytest

from conftest import gpu_available, rel_err, small_cases

pytestmark = pytest.mark.gpu

FIELDS = ["faceFD", "gradFD", "Flux", "Res", "FD", "cFD"]


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _bundle(name, fOrder):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    m, W, Wb, st = small_cases()[name]
    cfg = CaseConfig(stencilType=st, fOrder=fOrder, CFL=0.2 if name.startswith("ffs") else 0.5)
    return precompute(m, cfg, W, Wb, want_rbf64=True, gauss_flux=True), cfg


def test_one_point_rule_is_the_face_centre_flux():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = _bundle("mixed_riemann", 1)
    a = CudaSolver(hf, cfg, policy="fp64")
    b = CudaSolver(hf, cfg, policy="fp64", gauss_flux=True)
    dt = a.set_delta_t()
    for k in range(3):
        ra, rb = a.stage_debug(k, dt), b.stage_debug(k, dt)
        assert np.array_equal(ra["shockIndicator"], rb["shockIndicator"])
        scale = np.abs(ra["Flux"]).max()
        assert np.abs(ra["Flux"] - rb["Flux"]).max() <= 1e-12 * scale, k
        b.upload_state(FD=ra["FD"], cFD=ra["cFD"], cFDold=ra["cFD"] if k == 2 else None)
    a.close()
    b.close()


@pytest.mark.parametrize("name", ["mixed_riemann", "vortex_box", "ffs_tri"])
def test_fp64_multi_point_flux_matches_the_oracle(name):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver
    from oracle.oracle import Oracle

    hf, cfg = _bundle(name, 4)
    s = CudaSolver(hf, cfg, policy="fp64", gauss_flux=True)
    o = Oracle(hf, cfg.R, cfg.Cv, "fp64", gauss_flux=True)
    st = o.new_state()
    for step in range(2):
        dt = o.delta_t(st["FD"], cfg.CFL)
        assert s.set_delta_t() == pytest.approx(dt, rel=1e-13)
        for k in range(3):
            a = s.stage_debug(k, dt)
            c = o.stage(st, k, dt)
            assert np.array_equal(a["shockIndicator"], c["shockIndicator"]), f"flags differ step {step} stage {k}"
            for f in FIELDS:
                assert rel_err(a[f], c[f]) <= 1e-10, (f, step, k)
            s.upload_state(FD=c["FD"], cFD=c["cFD"], cFDold=c["cFD"] if k == 2 else None)
    s.close()


def test_mixed_multi_point_flux_close_to_fp64():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = _bundle("vortex_box", 4)
    a = CudaSolver(hf, cfg, policy="fp64", gauss_flux=True)
    b = CudaSolver(hf, cfg, policy="mixed", gauss_flux=True)
    a.run(20, dt=2e-2)
    b.run(20, dt=2e-2)
    assert a.launches_per_step() == 17 and b.launches_per_step() == 17
    ra, rb = a.state()["cFD"], b.state()["cFD"]
    assert np.isfinite(rb).all()
    scale = np.abs(ra).max(axis=0)
    assert (np.abs(ra - rb).max(axis=0) <= 1e-5 * scale).all()
    # the option changes the result: the face-centre flux on the same steps differs
    c = CudaSolver(hf, cfg, policy="fp64")
    c.run(20, dt=2e-2)
    assert np.abs(c.state()["cFD"] - ra).max() > 1e-8 * np.abs(ra).max()
    for x in (a, b, c):
        x.close()


def test_batch_refuses_a_solver_with_the_multi_point_flux():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, Batch, CudaSolver

    hf, cfg = _bundle("quad_riemann", 4)
    s = CudaSolver(hf, cfg, policy="mixed", gauss_flux=True)
    b = Batch("mixed")
    s.set_step_params()
    with pytest.raises(AfarError):
        b.add(s)
    s.set_face_gauss_flux(None)  # back to the face-centre flux: it may join
    b.add(s)
    b.run(2)
    b.close()
    s.close()
