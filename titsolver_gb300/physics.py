"""Parameter presets of the two term sets the GPU path implements.

* ``reference_params``: TitSolver's own FluidEquations terms
  (source/tit/sph/fluid_equations.hpp): Morris laminar viscosity mu, Ferrari
  density diffusion, CFL 0.4, C_force 0.25, C_visc 0.125 (:518-520), the C4
  Wendland kernel and mu = 0.001 of source/titwcsph/wcsph.cpp:52,89.
* ``baseline_params``: the textbook weakly-compressible set the dam-break
  benchmark names: Wendland C2, Monaghan artificial viscosity alpha = 0.02,
  delta-SPH (Molteni & Colagrossi) delta = 0.1, CFL 0.25, no laminar mu.
"""

from __future__ import annotations

from . import _abi


def reference_params(dim: int = 2, precision: int = _abi.TG_FP64,
                     kernel: int = _abi.TG_KERNEL_WENDLAND_C4) -> _abi.TgParams:
    p = _abi.TgParams()
    p.dim = dim
    p.precision = precision
    p.kernel = kernel
    p.integrator = _abi.TG_SSPRK3
    p.viscosity = _abi.TG_VISC_MORRIS
    p.diffusion = _abi.TG_DIFF_FERRARI
    p.post_integrate = _abi.TG_POST_PREPARE
    p.cells_per_radius = 2
    p.kahan = 1
    p.device = -1
    p.staging = 0
    p.resort = 1
    p.xi = 7.0
    p.g = 9.81
    p.mu = 0.001
    p.alpha = 0.0
    p.delta = 0.0
    p.cfl = 0.4
    p.c_force = 0.25
    p.c_visc = 0.125
    return p


def baseline_params(dim: int = 2, precision: int = _abi.TG_FP64,
                    kernel: int = _abi.TG_KERNEL_WENDLAND_C2) -> _abi.TgParams:
    p = reference_params(dim, precision, kernel)
    p.viscosity = _abi.TG_VISC_MONAGHAN
    p.diffusion = _abi.TG_DIFF_MOLTENI
    p.mu = 0.0
    p.alpha = 0.02
    p.delta = 0.1
    p.cfl = 0.25
    return p
