"""The reference's density-method SIMP samples (sample/optimize/sample_optimize_density_{oc,mma,
CONLIN}.cpp:23-204) as problem descriptions: the 60x40 cantilever, left edge clamped, unit
downward load at (60, 20), E1 = 210000, E0 = 1e-4, scale0 = 1e5, weight limit 0.5, filter radius
1.5, the Heaviside filter with beta doubled every 40 iterations from 0.5, and the samples'
optimiser settings; each runs until its optimiser's IsConvergence.  Values: (problem factory,
the VTK file the sample's last iteration left in the reference tree)."""
from pansfem2_gb300 import problems as PB

_COMMON = dict(E1=210000.0, E0=1e-4, scale0=1e5, vf=0.5, R=1.5, heaviside=1)

SAMPLES = {
    # OC(n, 0.5, 0.0, 1e4, 1e-3, 0.15, ...) (sample_optimize_density_oc.cpp:80)
    "oc": (lambda: PB.cantilever_q4(60, 40, optimizer=0, oc_move=0.15, **_COMMON), "Density_OC.vtk"),
    # MMA(n, 1, 1.0, {0}, {1e4}, {0}, 0.01, 1.0), SetParameters(1e-5, 0.1, 0.2, 0.5, 0.7, 1.2, 1e-6)
    # (sample_optimize_density_mma.cpp:80-85)
    "mma": (lambda: PB.cantilever_q4(60, 40, optimizer=1, mma_a0=1.0, mma_c=1e4, mma_d=0.0, mma_raa0=1e-5,
                                     mma_albefa=0.1, mma_move=0.2, mma_asyinit=0.5, mma_asydecr=0.7,
                                     mma_asyincr=1.2, mma_eps=1e-6, **_COMMON), "Density_MMA.vtk"),
    # CONLIN(n, 1, 1.0, {0}, {1e4}, {0}, 0.01, 1.0), SetParameters(0.2, 1e-6)
    # (sample_optimize_density_CONLIN.cpp:80-85)
    "conlin": (lambda: PB.cantilever_q4(60, 40, optimizer=2, mma_a0=1.0, mma_c=1e4, mma_d=0.0, mma_move=0.2,
                                        mma_eps=1e-6, **_COMMON), "Density_CONLIN.vtk"),
}
