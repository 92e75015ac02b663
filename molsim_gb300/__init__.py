"""molsim_gb300 — MOLSIM's force/energy hot path on one GB300 GPU.

The native library (libmolsim_gb300.so, built from csrc/ for sm_103a) holds
every kernel and the C ABI of include/molsim_gb300.h; this package is the
host-side mirror of the reference's interface (see engine.Engine) plus the
system description and seeded workloads.
"""
from . import abi, configs, units
from .engine import Engine, MolsimError
from .system import Species, System

__all__ = ["abi", "configs", "units", "Engine", "MolsimError", "Species", "System", "build"]


def build(verbose=False, force=False):
    """Compile the native library in place (nvcc, sm_103a) and the compiled
    ABI caller next to it (native_build.py)."""
    from .native_build import build as _b
    return _b(verbose=verbose, force=force)
