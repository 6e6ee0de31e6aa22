"""The ROM incompressible solver's implicit steps on the GPU: the HelmSolve callers of
VelocityCorrectionScheme_ROM (solvers/IncNavierStokesSolver/EquationSystems/
VelocityCorrectionScheme_ROM.cpp:1522-1567).

``VelocityCorrectionGPU.solve_viscous`` is ``v_SolveViscous``: every velocity field is one
Helmholtz solve with lambda = 1 / (aii_dt * diff_coeff[i]) followed by a BwdTrans of its
coefficients to the quadrature points. ``solve_pressure`` is ``v_SolvePressure``: the
pressure Poisson equation, HelmSolve with lambda = 0. The velocity fields share one
expansion, so one ``GlobalLinSysIterativeFullGPU`` serves them all; the pressure has its own.
"""
import ctypes

import numpy as np

from . import _capi as C
from .operators import _is_device, _like, _ptr, _same_side


def _ptr_array(arrays, dtype=None):
    """ctypes array of pointers to the given arrays (None -> NULL) and their on_device flag."""
    ptrs, sides = [], set()
    for a in arrays:
        if a is None:
            ptrs.append(None)
            continue
        p, d = _ptr(a, dtype)
        ptrs.append(p.value)
        sides.add(d)
    if len(sides) > 1:
        raise ValueError("the arrays of one call must be all host numpy arrays or all CUDA tensors")
    return (ctypes.c_void_p * len(ptrs))(*ptrs), (sides.pop() if sides else 1)


class VelocityCorrectionGPU:
    """The implicit steps of VelocityCorrectionScheme_ROM on GPU systems.

    velocity: GlobalLinSysIterativeFullGPU of the velocity expansion (shared by the fields);
    pressure: the pressure expansion's system (optional); diff_coeff: the diffusion
    coefficient of each velocity field (m_diffCoeff, the kinematic viscosity)."""

    def __init__(self, velocity, diff_coeff, pressure=None):
        self.velocity = velocity
        self.pressure = pressure
        self.diff_coeff = np.ascontiguousarray(diff_coeff, dtype=np.float64).reshape(-1)
        if self.diff_coeff.size == 0:
            raise ValueError("at least one velocity field")

    @property
    def nfields(self):
        return self.diff_coeff.size

    def solve_viscous(self, forcing, aii_dt, dirichlet=None, coeffs=None, phys=None, **kw):
        """v_SolveViscous: forcing[i] at the quadrature points -> coeffs[i] (local
        coefficients) and phys[i] = BwdTrans(coeffs[i]). dirichlet[i]: the field's ndir
        Dirichlet coefficients (None: homogeneous). Returns (coeffs, phys, [CgResult])."""
        nf = self.nfields
        if len(forcing) != nf:
            raise ValueError(f"expected {nf} forcing fields")
        sysg = self.velocity
        coll = sysg.coll
        nloc, nphys = coll.E * coll.nm, coll.E * coll.nq
        ref = forcing[0]
        coeffs = coeffs if coeffs is not None else [_like(ref, nloc) for _ in range(nf)]
        phys = phys if phys is not None else [_like(ref, nphys) for _ in range(nf)]
        dirs = list(dirichlet) if dirichlet is not None else [None] * nf
        if len(coeffs) != nf or len(phys) != nf or len(dirs) != nf:
            raise ValueError(f"expected {nf} entries per field list")
        _same_side(*forcing, *coeffs, *phys, *[d for d in dirs if d is not None])
        f_arr, dev = _ptr_array(forcing, None if _is_device(ref) else np.float64)
        c_arr, _ = _ptr_array(coeffs)
        p_arr, _ = _ptr_array(phys)
        d_arr = None
        if any(d is not None for d in dirs):
            d_arr, _ = _ptr_array(dirs, None if _is_device(ref) else np.float64)
        res = (C.CgResult * nf)()
        o = sysg.options(**kw)
        dc = self.diff_coeff
        C.call("ithaca_gpu_vcs_solve_viscous", sysg.handle, nf, f_arr, d_arr, ctypes.c_double(aii_dt),
               ctypes.c_void_p(dc.ctypes.data), c_arr, p_arr, ctypes.byref(o), res, dev)
        return coeffs, phys, list(res)

    def solve_pressure(self, forcing, dirichlet=None, out=None, **kw):
        """v_SolvePressure: the pressure Poisson equation (lambda = 0), forcing at the
        quadrature points -> local coefficients of the pressure expansion.
        Returns (coefficients, CgResult)."""
        if self.pressure is None:
            raise ValueError("no pressure system")
        sysg = self.pressure
        out = out if out is not None else _like(forcing, sysg.coll.E * sysg.coll.nm)
        _same_side(forcing, out, dirichlet)
        res = C.CgResult()
        o = sysg.options(**kw)
        pf, d = _ptr(forcing, np.float64 if not _is_device(forcing) else None)
        po, _ = _ptr(out)
        pd, _ = _ptr(dirichlet, np.float64 if not _is_device(forcing) else None)
        C.call("ithaca_gpu_vcs_solve_pressure", sysg.handle, pf, pd, po, ctypes.byref(o), ctypes.byref(res), d)
        return out, res
