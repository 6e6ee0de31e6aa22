"""Generates tests/golden/pyr.npz: pyramid fixtures from the reference's own code.

Run in the container that has the reference tree (after ``make -C oracle/ref``):
    python tests/golden/make_pyr_golden.py
Outputs come from oracle/_ref/libithaca_ref.so: Polylib's zwgrjm/Dgrjm (alpha 2), the
eModifiedPyr_C rows of Basis.cpp:568-672 and the MatrixFree pyramid kernel templates
(BwdTransPyrKernel, IProductPyrKernel, PhysDerivPyrKernel, PhysDerivTensor3DKernel)
compiled in place and composed as HelmholtzPyrImpl and IProductWRTDerivBasePyrImpl
compose them (oracle/ref/ref_kernels.cpp). Contents:
  * t{n}_*        direction-2 tables n = 2..10: z2 w2 D2 B2 DB2
  * unit_helm_*   the MatrixFree Helmholtz case of
                  library/UnitTests/Collections/TestPyrCollection.cpp:2653-2740 (the standard
                  pyramid, 4 modes, 10 elements, lambda 1.5, coefficients 1)
  * unit_bwd_*    BwdTrans of the same element (:2297-2380), coefficients 1
  * mesh_*        a curved, jittered 1 x 1 x 1 PyrMesh (6 pyramids, 5 modes), per-point
                  geometry: every operator on seeded inputs
  * reg_*         a straight unjittered 1 x 1 x 1 PyrMesh, per-element geometry, 4 modes
Geometry inputs come from the oracle's pyramid GeomFactors restatement.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu.mesh import PyrMesh  # noqa: E402
from oracle import pyr as opyr  # noqa: E402
from oracle import refbind  # noqa: E402


def main():
    out = {}
    for n in range(2, 11):
        for name, v in zip(("z2", "w2", "D2", "B2", "DB2"), refbind.pyr_tables(n)):
            out[f"t{n}_{name}"] = v
    n, E = 4, 10
    pb = opyr.PyrBasis(n)
    # the standard pyramid: x = xi, J = 1, df = identity
    J = np.ones(E)
    df = np.zeros((9, E))
    df[[0, 4, 8]] = 1.0
    out["unit_helm_jac"], out["unit_helm_df"], out["unit_helm_lambda"] = J, df, 1.5
    out["unit_helm_out"] = refbind.pyr_helmholtz(n, E, J, df, False, 1.5, np.ones(E * pb.nc))
    out["unit_bwd_out"] = refbind.pyr_bwdtrans(n, 1, np.ones(pb.nc))
    rng = np.random.default_rng(61)
    for tag, mesh, n, deformed in (("mesh", PyrMesh(1, 1, 1, jitter=0.0, seed=4, curve_amp=0.05), 5, True),
                                   ("reg", PyrMesh(1, 1, 1), 4, False)):
        pb = opyr.PyrBasis(n)
        E = mesh.E
        X = mesh.coords(n)
        J, df = opyr.geom_factors(pb, X)
        if not deformed:
            J, df = J[:, 0].copy(), df.reshape(9, E, -1)[:, :, 0].copy()
        u = rng.uniform(-1, 1, E * pb.nc)
        f, g, h = (rng.uniform(-1, 1, E * pb.nq) for _ in range(3))
        out.update({f"{tag}_n": n, f"{tag}_jac": J.reshape(-1), f"{tag}_df": df, f"{tag}_u": u, f"{tag}_f": f,
                    f"{tag}_g": g, f"{tag}_h": h,
                    f"{tag}_bwd": refbind.pyr_bwdtrans(n, E, u),
                    f"{tag}_iprod": refbind.pyr_iproduct(n, E, J.reshape(-1), deformed, f),
                    f"{tag}_deriv": np.stack(refbind.pyr_physderiv(n, E, df, deformed, f)),
                    f"{tag}_iprd": refbind.pyr_iproduct_deriv(n, E, J.reshape(-1), df, deformed, f, g, h),
                    f"{tag}_helm": refbind.pyr_helmholtz(n, E, J.reshape(-1), df, deformed, 1.3, u)})
    np.savez_compressed(os.path.join(HERE, "pyr.npz"), **out)
    print("pyr.npz written to", HERE)


if __name__ == "__main__":
    main()
