"""GB300-native WCSPH hot path of TitSolver: neighbour search, fused kernel
sums and the SSPRK integrator step as CUDA kernels for sm_103a, behind the C
ABI of ``include/titgpu.h``.  ``titsolver_gb300.sph`` mirrors the reference's
ParticleArray / FluidEquations / SSPRKIntegrator interface over that ABI."""

from . import scenarios  # noqa: F401

__all__ = ["scenarios"]
