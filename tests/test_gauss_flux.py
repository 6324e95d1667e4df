"""The optional multi-point face flux on the CPU: the Gauss-point O3 weights of the precompute and
the oracle's FP64 restatement of the option (the checker of the GPU kernels).  No GPU."""
import numpy as np
import pytest

from conftest import small_cases


@pytest.mark.parametrize("name", ["mixed_riemann", "ffs_tri", "vortex_box"])
def test_gauss_point_weights(name):
    """Every point's weights sum to one; the 1-point rule (the face centre) gives exactly the
    face-centre weights; the rest of the bundle does not change."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    m, W, Wb, st = small_cases()[name]
    for fOrder, ng in ((1, 1), (3, 2), (4, 3), (7, 4)):
        cfg = CaseConfig(stencilType=st, fOrder=fOrder)
        hf = precompute(m, cfg, W, Wb, want_rbf64=True, gauss_flux=True)
        nf, nmax = hf.nf, hf.sizes["maxStencilSize"] + 1
        g = hf.a["RBFbasisGauss64"].reshape(nf, 2, ng, nmax)
        assert hf.a["faceGaussPoints"].shape == (nf, ng, 2)
        np.testing.assert_allclose(g.sum(axis=3), 1.0, rtol=0, atol=1e-12)
        if ng == 1:
            assert np.array_equal(g[:, :, 0, :], hf.a["RBFbasis64"].reshape(nf, 2, nmax))
        plain = precompute(m, cfg, W, Wb, want_rbf64=True)
        for k in plain.a:
            assert np.array_equal(plain.a[k], hf.a[k]), k


def _stage(hf, cfg, gauss, k=0):
    from oracle.oracle import Oracle

    o = Oracle(hf, cfg.R, cfg.Cv, "fp64", gauss_flux=gauss)
    st = o.new_state()
    return o.stage(st, k, o.delta_t(st["FD"], cfg.CFL))


def test_oracle_one_point_rule_is_the_face_centre_flux():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    m, W, Wb, st = small_cases()["vortex_box"]
    cfg = CaseConfig(stencilType=st, fOrder=1)
    hf = precompute(m, cfg, W, Wb, want_rbf64=True, gauss_flux=True)
    a, b = _stage(hf, cfg, False), _stage(hf, cfg, True)
    assert np.abs(a["Flux"] - b["Flux"]).max() <= 1e-14 * np.abs(a["Flux"]).max()


def test_oracle_multi_point_flux_free_stream_and_conservation():
    """A uniform stream stays uniform (zero residual) and the residuals of all cells add up to the
    boundary fluxes (each internal face flux enters two cells with opposite signs)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    cfg = CaseConfig(stencilType="edgeNeighbour", fOrder=4)
    m = mesh.riemann_mixed(16, seed=3)
    W, Wb = mesh.uniform_fields(m, 1.0, 0.4, -0.3, 1.2)
    hf = precompute(m, cfg, W, Wb, want_rbf64=True, gauss_flux=True)
    r = _stage(hf, cfg, True)
    assert np.abs(r["Res"]).max() <= 1e-12
    m, W, Wb, st = small_cases()["vortex_box"]
    hf = precompute(m, CaseConfig(stencilType=st, fOrder=4), W, Wb, want_rbf64=True, gauss_flux=True)
    r = _stage(hf, CaseConfig(stencilType=st, fOrder=4), True)
    bsum = r["Flux"][hf.nf:].sum(axis=0)
    np.testing.assert_allclose(r["Res"].sum(axis=0), bsum, rtol=0, atol=1e-12 * np.abs(r["Flux"]).max())
    # on a smooth flow the points see the state's variation along the face: the flux differs
    a = _stage(hf, CaseConfig(stencilType=st, fOrder=4), False)
    assert np.abs(a["Flux"] - r["Flux"]).max() > 1e-4 * np.abs(a["Flux"]).max()
