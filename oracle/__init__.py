"""CPU oracle for the spectral/hp Helmholtz + CG + POD path (TEST INFRASTRUCTURE ONLY).

This package restates, in numpy, the FP64 arithmetic of the reference code path
(Nektar++ 5.0.0 as shipped in ITHACA-SEM) that the GPU library replaces:

* ``polylib``  -- Gauss-Lobatto-Legendre points/weights, collocation derivative
                  matrix, Jacobi polynomials (LibUtilities/Polylib/Polylib.cpp).
* ``basis``    -- the ModifiedA modal basis and its derivative
                  (LibUtilities/Foundations/Basis.cpp:392-421).
* ``geom``     -- Jacobian and derivative factors at quadrature points
                  (SpatialDomains/GeomFactors.cpp:168-475).
* ``ops``      -- BwdTrans / IProductWRTBase / PhysDeriv / Helmholtz on quads and
                  hexes, composed as MatrixFreeOps/Helmholtz.h:137-275,763-993.
* ``solve``    -- C0 gather/scatter, Jacobi diagonal, the reference's
                  single-reduction PCG (LibUtilities/LinearAlgebra/NekLinSysIterCG.cpp).
* ``pod``      -- method-of-snapshots POD, reduced operators and reduced solves
                  (solvers/IncNavierStokesSolver/EquationSystems/CoupledLinearNS_ROM.cpp).
* ``adjoint``  -- variable-coefficient Laplacian and the adjoint gradient.
* ``refbind``  -- ctypes binding of ``oracle/_ref/libithaca_ref.so``, which is
                  compiled from the reference's own Polylib.cpp and MatrixFreeOps
                  kernel headers by ``oracle/ref/Makefile``; it pins this restatement.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker. The GPU library
(``ithaca-sem_gb300``) never imports, links or executes anything here.
"""
