"""Generates the golden vectors in this directory: the reference's own CUDA kernels (cubins compiled
from its sources by oracle/build_ref.sh, launched by oracle/ref_harness.cpp) run on small seeded
meshes; every intermediate of one RK3 step is saved together with the exact inputs.

Run on a machine with a GPU and the cubins (output directory as the first argument):
    python tests/golden/make_golden.py tests/golden
The CPU tests (tests/test_golden.py) replay the saved inputs through the CPU oracle and compare.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

INPUTS = ["CELL", "FACE", "cellVolume", "neighbour", "boundaryFaceNeiLabel", "boundaryFacesType", "stencilSize",
          "compactStencilSize", "localStencil", "extendStencil", "cellFaces", "RBFbasis"]
OUTPUTS = ["faceFD", "gradFD", "limiter", "shockIndicator", "Flux", "Res", "FD", "cFD"]


def cases():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh

    out = {}
    m = mesh.quad_grid(16, 12, 0.0, 1.2, 0.0, 1.0)
    W, Wb = mesh.riemann_fields(m)
    out["quad_riemann_16x12"] = (m, W, Wb, CaseConfig(stencilType="faceNeighbour", CFL=0.3), 6)
    m = mesh.riemann_mixed(14, seed=7)
    W, Wb = mesh.riemann_fields(m)
    out["mixed_riemann_14"] = (m, W, Wb, CaseConfig(stencilType="edgeNeighbour", CFL=0.3), 6)
    return out


def main(outdir):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import precompute
    from oracle import ref_harness

    ref_harness.build()
    os.makedirs(outdir, exist_ok=True)
    for name, (m, W, Wb, cfg, presteps) in cases().items():
        hf = precompute(m, cfg, W, Wb)
        r = ref_harness.RefKernels(hf)
        for _ in range(presteps):  # develop shocks so that every switch branch is exercised
            r.evolve(1, cfg.R, cfg.Cv, r.adjust_dt(cfg.R, cfg.Cv, cfg.CFL))
        st = r.state()
        dt = r.adjust_dt(cfg.R, cfg.Cv, cfg.CFL)
        rec = {f"in_{k}": hf.a[k] for k in INPUTS}
        rec["in_matrix"] = st["matrix"]  # the LS rows the reference's calcLeastSquareMatrix built
        rec["in_FD"] = st["FD"]
        rec["in_cFD"] = st["cFD"]
        rec["sizes"] = np.array([hf.sizes[k] for k in ("cellsNum", "facesNum", "patchesNum", "totalBoundaryFacesNum",
                                                       "maxStencilSize", "maxCompactStencilSize",
                                                       "maxLocalBlockStencilSize",
                                                       "maxCompactLocalBlockStencilSize")], dtype=np.int64)
        rec["gas"] = np.array([cfg.R, cfg.Cv, cfg.CFL, dt])
        for k in range(3):
            o = r.stage(k, cfg.R, cfg.Cv, dt)
            for n in OUTPUTS:
                rec[f"stage{k}_{n}"] = o[n]
        np.savez_compressed(os.path.join(outdir, f"{name}.npz"), **rec)
        flags = rec["stage0_shockIndicator"][1::2]
        print(name, hf.nc, "cells, dt", dt, "switch counts", np.bincount(flags.astype(np.int64) + 2))
        r.close()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
