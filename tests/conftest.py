import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); compares the CUDA path with the oracles")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Compile libafar and the oracle once per session (incremental)."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import build

    build.build_all()
    return True


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def small_cases():
    """Seeded small meshes with their initial fields, sized for the oracle to finish in seconds."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh as M

    cases = {}
    m = M.quad_grid(24, 20, 0.0, 1.2, 0.0, 1.0)
    W, Wb = M.riemann_fields(m)
    cases["quad_riemann"] = (m, W, Wb, "faceNeighbour")
    m = M.forward_step_triangles(1500, seed=3)
    W, Wb = M.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
    cases["ffs_tri"] = (m, W, Wb, "edgeNeighbour")
    m = M.forward_step_triangles(1500, seed=4, renumber="hilbert")  # the benchmark's cell order
    W, Wb = M.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
    cases["ffs_tri_hilbert"] = (m, W, Wb, "edgeNeighbour")
    m = M.riemann_mixed(30, seed=5)
    W, Wb = M.riemann_fields(m)
    cases["mixed_riemann"] = (m, W, Wb, "edgeNeighbour")
    m = M.corner_flow(24)
    nb = m.n_boundary_faces
    # reference simulation/cornerFlow/cornerFlow_cuda/0/{p,U,T}: quiescent p=1, U=0, T=1; inlet fixed
    W = np.tile([1.0, 0.0, 0.0, 1.0], (m.n_cells, 1))
    Wb = np.tile([1.0, 0.0, 0.0, 1.0], (nb, 1))
    inlet = [p for p in m.patches if p[0] == "inlet"][0]
    Wb[inlet[2] - m.n_internal_faces: inlet[2] - m.n_internal_faces + inlet[3]] = [30.05945, 4.07795, 0.0, 5.97677]
    cases["corner_flow"] = (m, W, Wb, "edgeNeighbour")
    # the isentropic vortex (strength 5, free stream 1) on 20 x 20 quads of the [-7, 9]^2 box, outlets
    m = M.vortex_box(20)
    W = M.vortex_fields(m.cell_centres(), xc=0.0, yc=0.0)
    Wb = M.vortex_fields(m.boundary_face_centres(), xc=0.0, yc=0.0)
    cases["vortex_box"] = (m, W, Wb, "edgeNeighbour")
    return cases


def rel_err(a, b):
    """Max relative difference, scaled by max(|b|, 1e-3 max|b|); entries that are bit-identical
    (including matching NaNs) count as zero."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    if same.all():
        return 0.0
    finite = np.abs(b[np.isfinite(b)])
    bmax = finite.max() if finite.size else 0.0
    scale = np.maximum(np.abs(b), bmax * 1e-3 + 1e-300)
    d = np.where(same, 0.0, np.abs(a - b) / scale)
    return float(np.nanmax(np.where(np.isnan(d), np.inf, d)))


VORTEX_T_END = 2.0


def vortex_case(n, cfg, want_rbf64=False):
    """The isentropic vortex on n x n quads of the [-7, 9]^2 box: mesh, Gauss rules, initial cell
    averages (conserved U0, primitive W0), boundary ghosts Wb and the precomputed host fields."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import gauss_quadrature, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh as M

    m = M.vortex_box(n)
    quad = gauss_quadrature(m, cfg)
    U0 = M.vortex_cell_averages(m, quad, 0.0)
    W0 = M.primitive_from_conserved(U0)
    Wb = M.vortex_fields(m.boundary_face_centres(), xc=0.0, yc=0.0)
    hf = precompute(m, cfg, W0, Wb, want_rbf64=want_rbf64)
    return m, quad, U0, W0, Wb, hf


def vortex_l1(m, quad, rho, t=VORTEX_T_END):
    """Area-weighted L1 error of the density cell averages against the exact solution at t."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh as M

    exact = M.vortex_cell_averages(m, quad, t)[:, 0]
    area = m.cell_areas()
    return float(np.sum(np.abs(rho - exact) * area) / np.sum(area))


def oracle_vortex(n, cfg, policy="fp64"):
    """The CPU oracle's run of the vortex to VORTEX_T_END: (final state, steps, L1 error)."""
    from oracle.oracle import Oracle

    m, quad, U0, W0, Wb, hf = vortex_case(n, cfg, want_rbf64=policy == "fp64")
    o = Oracle(hf, cfg.R, cfg.Cv, policy)
    st = {"FD": np.concatenate([W0, Wb]), "cFD": U0.copy(), "cFDold": U0.copy(),
          "si": np.zeros(2 * (hf.nc + hf.nb), dtype=np.int8)}
    t, steps = 0.0, 0
    while t < VORTEX_T_END:
        dt = min(o.delta_t(st["FD"], cfg.CFL), VORTEX_T_END - t)
        o.evolve(st, dt)
        t += dt
        steps += 1
    return st, steps, vortex_l1(m, quad, st["cFD"][:, 0])
