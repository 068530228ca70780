"""GB300-native (sm_103a) parametric light-curve fitting.

The fused fit of the reference's per-band parametric path (PSO model selection
over the flux models, L-BFGS polish, SVI or Laplace uncertainty, profile
refinements, MultiBazin) runs as hand-written CUDA kernels in
``liblcf_gb300.so`` behind the C ABI declared in include/lcf.h.
"""
from . import abi, synth  # noqa: F401

__all__ = ["abi", "synth"]
