"""Periodic meshes (no boundary faces; the two sides of each period meet in internal faces): the
mesh generator, and a precompute that sees no seam: on a uniform periodic grid every cell has the
same stencil size and every face of one orientation the same O3 weights, seam faces included."""
import numpy as np
import pytest


@pytest.mark.parametrize("stencil,size", [("faceNeighbour", 12), ("edgeNeighbour", 8)])
def test_periodic_grid_has_no_seam(stencil, size):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    m = mesh.periodic_quad_grid(16, 12, 0.0, 1.6, 0.0, 1.2)
    assert m.n_boundary_faces == 0 and m.n_internal_faces == 2 * 16 * 12 and m.period == (1.6, 1.2)
    W = np.tile([1.0, 1.0, 0.5, 1.4], (m.n_cells, 1))
    hf = precompute(m, CaseConfig(stencilType=stencil), W, None, want_rbf64=True)
    assert hf.nb == 0 and hf.period == (1.6, 1.2)
    assert set(np.unique(hf.stencilSize)) == {size} and set(np.unique(hf.compactStencilSize)) == {4}
    r = hf.RBFbasis64.reshape(hf.nf, 2, -1)
    sfx = np.abs(np.round(hf.FACE[:, 3], 9))
    for orient in np.unique(sfx):
        w = np.sort(r[sfx == orient].reshape((sfx == orient).sum(), -1), axis=1)
        assert np.abs(w - w[0]).max() < 1e-9


def test_periodic_cell_averages_wrap():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, gauss_quadrature, mesh

    m = mesh.periodic_quad_grid(32, 32, 0.0, 10.0, 0.0, 10.0)
    q = gauss_quadrature(m, CaseConfig())
    a = mesh.vortex_cell_averages(m, q, 0.0, centre=(5.0, 5.0))
    b = mesh.vortex_cell_averages(m, q, 10.0, centre=(5.0, 5.0))  # one full period later: same field
    assert np.abs(a - b).max() < 1e-12


def test_wedge_mesh_patches():
    """The compression ramp of the batched workload: label-6 inflow, outlet, slip walls."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    m = mesh.wedge_quads(40, 20, 15.0)
    assert [(p[0], p[1], p[3]) for p in m.patches] == [("inflow", 6, 20), ("outflow", 4, 20), ("walls", 2, 80)]
    assert (m.cell_areas() > 0).all()
    W = mesh.vortex_fields(m.cell_centres(), strength=2.0, xc=0.5, yc=0.6, u0=3.0, v0=0.0)
    Wb = mesh.vortex_fields(m.boundary_face_centres(), strength=0.0, xc=0.5, yc=0.6, u0=3.0, v0=0.0)
    hf = precompute(m, CaseConfig(stencilType="faceNeighbour"), W, Wb)
    assert set(np.unique(hf.boundaryFacesType)) == {2, 4, 6}
