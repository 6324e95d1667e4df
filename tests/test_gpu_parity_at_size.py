"""Parity at the benchmark sizes, through the C ABI:

* the ref policy against the reference's own kernels (oracle/_ref cubins), stage by stage for one
  RK3 step from identical inputs, on the 2.0M-triangle Mach 3 step mesh (stencils up to 17) and the
  4.0M-cell mixed quad/triangle Riemann mesh (quads and triangles, stencils up to 15): every
  intermediate within 1e-12 relative and identical troubled-cell / switch flags;
* the fp64 policy against the CPU oracle (FP64 restatement) for one stage on the 2.0M mesh: 1e-10;
* the mixed policy's tile-staged reconstruct (four-face path, stencils up to 15) on the 4.0M mesh
  against the fp64 policy and against its register-pass variant, one stage each.

These are the sizes the benchmark runs; the small-mesh tests in test_gpu_parity.py cover more
stages and steps.  The meshes are built once per module (about half a minute each on the host).
"""
import numpy as np
import pytest

from conftest import gpu_available, rel_err

pytestmark = pytest.mark.gpu

REF_TOL = 1e-12
FIELDS = ["faceFD", "gradFD", "Flux", "Res", "FD", "cFD"]


def _case(kind):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    if kind == "step":  # the benchmark's workload: ~1M jittered points, RCM order, CFL 0.2
        m = mesh.forward_step_triangles(1_000_000, seed=0)
        W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
        cfg = CaseConfig(stencilType="edgeNeighbour", CFL=0.2)
    else:  # the 4M-cell mixed quad/triangle Riemann problem
        m = mesh.riemann_mixed(1766, seed=0)
        W, Wb = mesh.riemann_fields(m)
        cfg = CaseConfig(stencilType="edgeNeighbour", CFL=0.3)
    return precompute(m, cfg, W, Wb, want_rbf64=True, device=0), cfg


@pytest.fixture(scope="module")
def step_case():
    if not gpu_available():
        pytest.skip("no CUDA device")
    return _case("step")


@pytest.fixture(scope="module")
def mixed_case():
    if not gpu_available():
        pytest.skip("no CUDA device")
    return _case("riemann_mixed")


@pytest.fixture(scope="module")
def ref_kernels():
    from oracle import ref_harness

    ref_harness.build()
    if not ref_harness.available():
        pytest.skip("reference cubins not built (oracle/build_ref.sh needs the reference sources)")
    return ref_harness


def _ref_vs_reference_one_step(hf, cfg, ref_kernels, min_flags):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    s = CudaSolver(hf, cfg, policy="ref")
    r = ref_kernels.RefKernels(hf)
    # a few steps of the reference first, so the stages see a state with structure (the impulsive
    # start is uniform away from the walls); both sides then start each stage from its state
    for _ in range(3):
        r.evolve(1, cfg.R, cfg.Cv, r.adjust_dt(cfg.R, cfg.Cv, cfg.CFL))
    st = r.state()
    s.upload_state(FD=st["FD"], cFD=st["cFD"], cFDold=st["cFD"])
    dt = r.adjust_dt(cfg.R, cfg.Cv, cfg.CFL)
    assert abs(s.set_delta_t() - dt) <= 1e-15 * dt
    flags = 0
    for k in range(3):
        a = s.stage_debug(k, dt)
        b = r.stage(k, cfg.R, cfg.Cv, dt)
        assert np.array_equal(a["shockIndicator"], b["shockIndicator"]), f"flags differ at stage {k}"
        assert np.array_equal(a["limiter"], b["limiter"]), f"limiter differs at stage {k}"
        for f in FIELDS:
            e = rel_err(a[f], b[f])
            assert e <= REF_TOL, f"{f} differs by {e:.3e} at stage {k}"
        flags += int(np.count_nonzero(b["shockIndicator"]))
        s.upload_state(FD=b["FD"], cFD=b["cFD"], cFDold=b["cFD"] if k == 2 else None)
    s.close()
    r.close()
    assert flags >= min_flags, f"only {flags} switch decisions were exercised"


def test_ref_policy_matches_reference_kernels_on_the_2M_step_mesh(step_case, ref_kernels):
    hf, cfg = step_case
    assert hf.nc > 1_900_000 and hf.sizes["maxStencilSize"] >= 16
    _ref_vs_reference_one_step(hf, cfg, ref_kernels, min_flags=100)


def test_ref_policy_matches_reference_kernels_on_the_4M_mixed_mesh(mixed_case, ref_kernels):
    hf, cfg = mixed_case
    assert hf.nc > 3_900_000 and hf.sizes["maxCompactStencilSize"] == 4 and hf.sizes["maxStencilSize"] >= 15
    _ref_vs_reference_one_step(hf, cfg, ref_kernels, min_flags=1000)


def test_fp64_policy_matches_the_oracle_for_one_stage_on_the_2M_step_mesh(step_case):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver
    from oracle.oracle import Oracle

    hf, cfg = step_case
    s = CudaSolver(hf, cfg, policy="fp64")
    o = Oracle(hf, cfg.R, cfg.Cv, "fp64")
    st = o.new_state()
    dt = o.delta_t(st["FD"], cfg.CFL)
    assert s.set_delta_t() == pytest.approx(dt, rel=1e-13)
    a = s.stage_debug(0, dt)
    c = o.stage(st, 0, dt)
    assert np.array_equal(a["shockIndicator"], c["shockIndicator"])
    for f in FIELDS:
        assert rel_err(a[f], c[f]) <= 1e-10, f
    assert rel_err(s.limiter64(), c["limiter"]) <= 1e-10
    s.close()


def test_mixed_tile_reconstruct_on_the_4M_mixed_mesh(mixed_case):
    """The four-face tile path with stencils up to 15: one stage against the fp64 policy and
    against the register-pass reconstruct, both to FP32 rounding (the mixed policy reconstructs and
    forms fluxes in FP32)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = mixed_case
    f = CudaSolver(hf, cfg, policy="fp64")
    dt = f.set_delta_t()
    ref = f.stage_debug(0, dt)
    f.close()
    outs = []
    for variant in (0, 1):  # tile-staged, register pass
        m = CudaSolver(hf, cfg, policy="mixed")
        m.set_tuning(variant)
        outs.append(m.stage_debug(0, dt))
        m.close()
    tile, reg = outs
    nc = hf.nc
    # the face values and gradients of the FP32 reconstruction, to its rounding
    for k, tol in (("faceFD", 2e-5), ("gradFD", 2e-4)):
        scale = np.abs(ref[k]).max(axis=0) + 1e-30
        assert (np.abs(tile[k] - ref[k]).max(axis=0) <= tol * scale).all(), k
        assert (np.abs(tile[k] - reg[k]).max(axis=0) <= tol * scale).all(), k
    # switch decisions: the troubled-cell tests sit on thresholds, so a handful may flip in FP32
    flips = np.count_nonzero(tile["shockIndicator"][0:2 * nc:2] != ref["shockIndicator"][0:2 * nc:2])
    assert flips <= 1e-4 * nc, flips
    scale = np.abs(ref["cFD"]).max(axis=0)
    assert (np.abs(tile["cFD"] - ref["cFD"]).max(axis=0) <= 1e-5 * scale).all()
