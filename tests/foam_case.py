"""A small OpenFOAM case written by the tests: the Mach 3 forward-facing step (channel [0,3]x[0,1],
step [0.6,3]x[0,0.2] removed) as three hex blocks, inflow label 3, outflow label 4, slip walls."""
import os

HEADER = "FoamFile\n{\n    version 2.0;\n    format ascii;\n    class dictionary;\n    object %s;\n}\n"

BLOCK_MESH = """convertToMeters 1;
vertices
(
    (0 0 0) (0.6 0 0) (0.6 0.2 0) (0 0.2 0) (0 1 0) (0.6 1 0) (3 0.2 0) (3 1 0)
    (0 0 0.1) (0.6 0 0.1) (0.6 0.2 0.1) (0 0.2 0.1) (0 1 0.1) (0.6 1 0.1) (3 0.2 0.1) (3 1 0.1)
);
blocks
(
    hex (0 1 2 3 8 9 10 11) (%(na)d %(nb)d 1) simpleGrading (1 1 1)
    hex (3 2 5 4 11 10 13 12) (%(na)d %(nc)d 1) simpleGrading (1 1 1)
    hex (2 6 7 5 10 14 15 13) (%(nd)d %(nc)d 1) simpleGrading (1 1 1)
);
edges ();
boundary
(
    inflow { type patch; faces ( (0 3 11 8) (3 4 12 11) ); }
    outflow { type patch; faces ( (6 7 15 14) ); }
    walls
    {
        type patch;
        faces ( (0 1 9 8) (1 2 10 9) (2 6 14 10) (4 5 13 12) (5 7 15 13) );
    }
);
"""

SCHEMES = """gaussQuadrature { cOrder 5; fOrder 4; }
CUDA
{
    R 0.714285714285714;
    Cv 1.785714285714286;
    stencilType edgeNeighbour;
%(recalc)s    boundary { patch0 3; patch1 4; patch2 2; }   // inflow, outflow, walls
}
ddtSchemes { default Euler; }
"""

CONTROL = """application cudaEuler2DmixO3RK3solver;
startTime 0;
endTime %(end)g;
deltaT 0.0001;
writeControl adjustableRunTime;
writeInterval %(wi)g;
adjustTimeStep yes;
maxCo 0.2;
maxDeltaT 1;
"""

FIELD = """dimensions %(dims)s;
internalField uniform %(val)s;
boundaryField
{
    inflow { type fixedValue; value uniform %(val)s; }
    outflow { type zeroGradient; }
    walls { type %(wall)s; }
    defaultFaces { type empty; }
}
"""


def write_case(root, n=4, end=0.02, wi=0.005, recalc_basis=None, write_format=None):
    """Blocks of (3n x n), (3n x 4n), (12n x 4n) cells; write_format: the controlDict writeFormat."""
    for d in ("system", "0", "constant"):
        os.makedirs(os.path.join(root, d), exist_ok=True)

    def put(rel, obj, body):
        with open(os.path.join(root, rel), "w") as f:
            f.write(HEADER % obj + "\n" + body)

    put("system/blockMeshDict", "blockMeshDict", BLOCK_MESH % {"na": 3 * n, "nb": n, "nc": 4 * n, "nd": 12 * n})
    recalc = "" if recalc_basis is None else f"    recalcBasis {'true' if recalc_basis else 'false'};\n"
    put("system/fvSchemes", "fvSchemes", SCHEMES % {"recalc": recalc})
    put("system/controlDict", "controlDict",
        CONTROL % {"end": end, "wi": wi} + (f"writeFormat {write_format};\n" if write_format else ""))
    put("0/p", "p", FIELD % {"dims": "[1 -1 -2 0 0 0 0]", "val": "1", "wall": "zeroGradient"})
    put("0/U", "U", FIELD % {"dims": "[0 1 -1 0 0 0 0]", "val": "(3 0 0)", "wall": "slip"})
    put("0/T", "T", FIELD % {"dims": "[0 0 0 1 0 0 0]", "val": "1", "wall": "zeroGradient"})
    return root
