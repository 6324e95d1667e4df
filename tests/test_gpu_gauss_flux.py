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
                if f == "Res":  # a sum of fluxes: near a uniform state it is rounding noise, so scale by the fluxes
                    assert np.abs(a[f] - c[f]).max() <= 1e-10 * np.abs(c["Flux"]).max(), (f, step, k)
                else:
                    assert rel_err(a[f], c[f]) <= 1e-10, (f, step, k)
            s.upload_state(FD=c["FD"], cFD=c["cFD"], cFDold=c["cFD"] if k == 2 else None)
    s.close()


def test_mixed_multi_point_flux_close_to_fp64():
    """The mixed policy's multi-point flux against the fp64 policy's over 20 steps: the area-weighted
    L1 of the density difference is of the order the face-centre flux shows between the two policies
    (FP32 reconstruction and fluxes; switch decisions near thresholds may flip)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = _bundle("vortex_box", 4)
    V = hf.cellVolume

    def l1(x, y):
        return float(np.sum(np.abs(x[:, 0] - y[:, 0]) * V) / np.sum(V))

    out = {}
    for gauss in (True, False):
        for pol in ("fp64", "mixed"):
            s = CudaSolver(hf, cfg, policy=pol, gauss_flux=gauss)
            s.run(20, dt=2e-2)
            assert s.launches_per_step() == (17 if gauss else 13)
            out[gauss, pol] = s.state()["cFD"]
            assert np.isfinite(out[gauss, pol]).all()
            s.close()
    d_gauss = l1(out[True, "mixed"], out[True, "fp64"])
    d_centre = l1(out[False, "mixed"], out[False, "fp64"])
    assert d_gauss <= max(1e-5, 3.0 * d_centre), (d_gauss, d_centre)
    # the option changes the result: the face-centre flux on the same steps differs
    assert l1(out[True, "fp64"], out[False, "fp64"]) > 1e-8


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
