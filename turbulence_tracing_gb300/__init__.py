"""turbulence_tracing_gb300 -- GB300 (sm_103a) implementation of the ray-integration
path of jdhare/turbulence_tracing.

Drop-in modules (same names and call signatures as the reference):
  particle_tracker     ElectronCube, dsdt
  ray_transfer_matrix  matrices, filters, Shadowgraphy / Schlieren_DF / Schlieren_LF / AFR
  turboGen             gaussian3D_FFT
Device-level API: core (torch CUDA tensors in and out).
Native code: libturbotrace.so (include/turbotrace.h), built by build.build().
"""
from . import build  # noqa: F401

__all__ = ["particle_tracker", "ray_transfer_matrix", "turboGen", "core", "build"]


def __getattr__(name):
    if name in ("particle_tracker", "ray_transfer_matrix", "turboGen", "core"):
        import importlib

        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
