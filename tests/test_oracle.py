"""Properties of the CPU oracle that hold for the reference algorithm itself (no GPU):
free-stream preservation, flux consistency of Roe and KFVS, discrete conservation of the signed
residual gather, the BC table, the CFL step, and the RK3 coefficients."""
import numpy as np
import pytest

from conftest import small_cases


@pytest.fixture(scope="module")
def cases():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    out = {}
    for name, (m, W, Wb, st) in small_cases().items():
        cfg = CaseConfig(stencilType=st)
        out[name] = (m, precompute(m, cfg, W, Wb, want_rbf64=True), cfg)
    return out


def _uniform(hf, W0):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import precompute  # noqa: F401

    FD = np.tile(W0, (hf.nc + hf.nb, 1)).astype(np.float64)
    return FD


def _euler_flux(W, S, R, Cv):
    p, ux, uy, T = W
    rho = p / (R * T)
    un = ux * S[:, 0] + uy * S[:, 1]
    F = np.stack([rho * un, rho * un * ux + p * S[:, 0], rho * un * uy + p * S[:, 1],
                  rho * un * (Cv * T + 0.5 * (ux * ux + uy * uy) + p / rho)], axis=1)
    return F


@pytest.mark.parametrize("policy", ["ref", "fp64"])
@pytest.mark.parametrize("name", ["quad_riemann", "ffs_tri", "mixed_riemann"])
def test_free_stream_preservation(cases, name, policy):
    from oracle.oracle import Oracle

    m, hf, cfg = cases[name]
    o = Oracle(hf, cfg.R, cfg.Cv, policy)
    st = o.new_state()
    W0 = np.array([1.3, 0.7, -0.4, 1.1])
    st["FD"][:] = W0
    # boundary ghosts equal to the interior state: outflow everywhere is preserved
    r = o.stage(st, 0, 1e-3)
    scale = np.abs(r["Flux"]).max()
    bflux = r["Flux"][hf.nf:]
    # interior cells feel no net flux, to the precision of the staged stencil values (the reference
    # stages float copies, cudaLimiter.h:95-98; corner cells switch to double TVD states)
    interior = np.ones(hf.nc, bool)
    interior[hf.boundaryFaceNeiLabel] = False
    tol = 1e-6 if policy == "ref" else 1e-12
    assert np.abs(r["Res"][interior]).max() <= tol * scale
    assert np.all(r["shockIndicator"][0::2] == 0)
    np.testing.assert_allclose(bflux, _euler_flux(W0, hf.FACE[hf.nf:, 3:5], cfg.R, cfg.Cv), rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("policy,tol", [("ref", 2e-6), ("fp64", 1e-13)])
@pytest.mark.parametrize("shock", [False, True])
def test_flux_consistency(cases, policy, tol, shock):
    """F(W, W) is the Euler flux for Roe (dissipation vanishes) and for KFVS (half-range moments
    add up to the full Maxwellian moments)."""
    from oracle.oracle import Oracle, _ptr, lib
    import ctypes as C

    m, hf, cfg = cases["mixed_riemann"]
    o = Oracle(hf, cfg.R, cfg.Cv, policy)
    W0 = np.array([0.8, 1.7, -0.9, 1.3])
    FD = _uniform(hf, W0)
    grad = np.zeros((hf.nc, 8))
    lim = np.ones((hf.nc, 4), dtype=o.lim_dtype())
    fv = np.tile(W0, (2 * hf.nf, 1))
    si = np.zeros(2 * (hf.nc + hf.nb), dtype=np.int8)
    if shock:
        si[1:2 * hf.nc:2] = -2
    flux = np.zeros((hf.nf + hf.nb, 4))
    getattr(lib(), f"oracle_flux_{policy}")(C.byref(o.m), _ptr(FD), _ptr(grad), _ptr(lim), _ptr(fv), _ptr(si),
                                            cfg.R, cfg.Cv, _ptr(flux))
    exact = _euler_flux(W0, hf.FACE[:, 3:5], cfg.R, cfg.Cv)
    scale = np.abs(exact).max()
    assert np.abs(flux - exact).max() <= tol * scale


def test_residual_gather_conserves(cases):
    """Sum of the residuals = sum of the boundary fluxes (internal faces cancel)."""
    from oracle.oracle import Oracle

    m, hf, cfg = cases["quad_riemann"]
    o = Oracle(hf, cfg.R, cfg.Cv, "ref")
    st = o.new_state()
    r = o.stage(st, 0, 1e-4)
    total = r["Res"].sum(axis=0)
    bnd = r["Flux"][hf.nf:].sum(axis=0)
    np.testing.assert_allclose(total, bnd, rtol=1e-12, atol=1e-12 * np.abs(r["Flux"]).max())
    assert np.count_nonzero(r["shockIndicator"][1::2] < 0) > 0, "the Riemann case exercises KFVS faces"


def test_boundary_table():
    """cudaEulerBCs labels 0-5 (BCs/2D/*.h:4-10)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute
    from oracle.oracle import Oracle, _ptr, lib
    import ctypes as C

    m = mesh.quad_grid(3, 3)
    W, Wb = mesh.uniform_fields(m, 1.0, 0.0, 0.0, 1.0)
    hf = precompute(m, CaseConfig(stencilType="faceNeighbour"), W, Wb)
    Wc = np.array([2.0, 0.3, -0.7, 1.5])
    expect = {
        0: lambda n: [2.0, 0.0, 0.0, 1.0],
        1: lambda n: [2.0, 0.0, 0.0, 1.5],
        2: lambda n: [2.0, 0.3 - (0.3 * n[0] - 0.7 * n[1]) * n[0], -0.7 - (0.3 * n[0] - 0.7 * n[1]) * n[1], 1.5],
        3: lambda n: [1.0, 3.0, 0.0, 1.0],
        4: lambda n: [2.0, 0.3, -0.7, 1.5],
        5: lambda n: [30.05945, 4.07795, 0.0, 5.97677],
    }
    for label, fn in expect.items():
        hf.a["boundaryFacesType"][:] = label
        o = Oracle(hf, 1 / 1.4, 1 / 1.4 / 0.4)
        FD = np.tile(Wc, (hf.nc + hf.nb, 1))
        lib().oracle_boundary(C.byref(o.m), _ptr(FD), o.R, o.Cv)
        for b in range(hf.nb):
            S = hf.FACE[hf.nf + b, 3:5] / hf.FACE[hf.nf + b, 2]
            np.testing.assert_allclose(FD[hf.nc + b], fn(S), rtol=1e-15, atol=1e-15)


def test_cfl_step_formula(cases):
    """setDeltaT: CFL dR |S| / ((1-f)|U_L.S| + f|U_R.S| + c_f |S|), min with 1e5."""
    from oracle.oracle import Oracle

    m, hf, cfg = cases["ffs_tri"]
    o = Oracle(hf, cfg.R, cfg.Cv)
    FD = hf.FD.copy()
    dt = o.delta_t(FD, 0.5)
    nb = hf.neighbour.reshape(-1, 2)
    X = hf.CELL
    own, nei = nb[:, 0], nb[:, 1]
    dR = np.hypot(*(X[nei] - X[own]).T)
    fr = np.hypot(*(hf.FACE[:hf.nf, :2] - X[own]).T) / dR
    S = hf.FACE[:hf.nf, 3:5]
    mS = hf.FACE[:hf.nf, 2]
    un = lambda W: np.abs(W[:, 1] * S[:, 0] + W[:, 2] * S[:, 1])
    c = np.sqrt((cfg.R / cfg.Cv + 1) * cfg.R * ((1 - fr) * FD[own, 3] + fr * FD[nei, 3]))
    ref = np.min(0.5 * dR * mS / ((1 - fr) * un(FD[own]) + fr * un(FD[nei]) + c * mS))
    assert dt == pytest.approx(min(ref, 1e5), rel=1e-13)


def test_rk3_uses_reference_coefficients(cases):
    """GPUevolve.cu:223-225: beta = {1,0,1}, {0.75,0.25,0.25}, {0.333333,0.666667,0.666667}; with a
    zero residual the truncated decimals show up as the factor 0.333333 + 0.666667 = 1 exactly."""
    from oracle.oracle import Oracle

    assert Oracle.BETA[2] == (0.333333, 0.666667, 0.666667)
    m, hf, cfg = cases["mixed_riemann"]
    o = Oracle(hf, cfg.R, cfg.Cv, "fp64")
    st = o.new_state()
    st2 = o.new_state()
    o.evolve(st, 1e-4)
    o.evolve(st2, 1e-4, exact_rk=True)
    d = np.abs(st["cFD"] - st2["cFD"]).max()
    assert 0 < d < 1e-5
