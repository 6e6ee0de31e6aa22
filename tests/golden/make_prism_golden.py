"""Generates tests/golden/prism.npz: prism fixtures from the reference's own code.

Run in the container that has the reference tree (after ``make -C oracle/ref``):
    python tests/golden/make_prism_golden.py
Outputs come from oracle/_ref/libithaca_ref.so: the MatrixFree prism kernel templates
(BwdTransPrismKernel, IProductPrismKernel, PhysDerivPrismKernel, PhysDerivTensor3DKernel)
compiled in place and composed as HelmholtzPrismImpl and IProductWRTDerivBasePrismImpl
compose them (oracle/ref/ref_kernels.cpp); the tables are those of the triangle fixtures
(GLL + eModified_A in directions 0 and 1, Gauss-Radau + eModified_B in direction 2).
Contents:
  * unit_helm_*   the MatrixFree Helmholtz case of
                  library/UnitTests/Collections/TestPrismCollection.cpp:2946-3056 (the standard
                  prism, 6 modes, 10 elements, lambda 0, coefficients 1)
  * unit_bwd_*    BwdTrans of the same element (:373-462), coefficients 1
  * mesh_*        a curved, jittered 1 x 2 x 1 PrismMesh (4 prisms, 5 modes), per-point
                  geometry: every operator on seeded inputs
  * reg_*         a straight unjittered 2 x 1 x 1 PrismMesh, per-element geometry, 4 modes
Geometry inputs come from the oracle's prism GeomFactors restatement.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu.mesh import PrismMesh  # noqa: E402
from oracle import prism as oprism  # noqa: E402
from oracle import refbind  # noqa: E402


def main():
    out = {}
    n, E = 6, 10
    pb = oprism.PrismBasis(n)
    # the standard prism: x = xi, J = 1, df = identity
    J = np.ones(E)
    df = np.zeros((9, E))
    df[[0, 4, 8]] = 1.0
    out["unit_helm_jac"], out["unit_helm_df"], out["unit_helm_lambda"] = J, df, 0.0
    out["unit_helm_out"] = refbind.prism_helmholtz(n, E, J, df, False, 0.0, np.ones(E * pb.nc))
    out["unit_bwd_out"] = refbind.prism_bwdtrans(n, 1, np.ones(pb.nc))
    rng = np.random.default_rng(51)
    for tag, mesh, n, deformed in (("mesh", PrismMesh(1, 2, 1, jitter=0.2, seed=4, curve_amp=0.05), 5, True),
                                   ("reg", PrismMesh(2, 1, 1), 4, False)):
        pb = oprism.PrismBasis(n)
        E = mesh.E
        X = mesh.coords(n)
        J, df = oprism.geom_factors(pb, X)
        if not deformed:
            J, df = J[:, 0].copy(), df.reshape(9, E, -1)[:, :, 0].copy()
        u = rng.uniform(-1, 1, E * pb.nc)
        f, g, h = (rng.uniform(-1, 1, E * pb.nq) for _ in range(3))
        out.update({f"{tag}_n": n, f"{tag}_jac": J.reshape(-1), f"{tag}_df": df, f"{tag}_u": u, f"{tag}_f": f,
                    f"{tag}_g": g, f"{tag}_h": h,
                    f"{tag}_bwd": refbind.prism_bwdtrans(n, E, u),
                    f"{tag}_iprod": refbind.prism_iproduct(n, E, J.reshape(-1), deformed, f),
                    f"{tag}_deriv": np.stack(refbind.prism_physderiv(n, E, df, deformed, f)),
                    f"{tag}_iprd": refbind.prism_iproduct_deriv(n, E, J.reshape(-1), df, deformed, f, g, h),
                    f"{tag}_helm": refbind.prism_helmholtz(n, E, J.reshape(-1), df, deformed, 1.3, u)})
    np.savez_compressed(os.path.join(HERE, "prism.npz"), **out)
    print("prism.npz written to", HERE)


if __name__ == "__main__":
    main()
