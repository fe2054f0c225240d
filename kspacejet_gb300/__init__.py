"""GB300-native non-Cartesian reconstruction for KSpaceJet.

The product is native code (``kspacejet_gb300/lib``):

* ``libksj_gpu.so`` -- sm_103a kernels behind the C ABI ``include/ksj_gpu.h``;
* ``libksj_gb300_noncartesian_recon.so`` / ``libksj_gb300_coil_combine.so`` --
  drop-in Provider plug-ins exporting ``ksj_provider_query``
  (``include/ksj_provider_abi.h``);
* ``libksj_firing_host.so`` -- a synchronous Provider host.

This Python package only loads them (``gpu``, ``host``) and provides seeded
synthetic inputs (``synth``).  There is no CPU implementation of the
reconstruction anywhere in it: a missing library or device raises.
"""
from __future__ import annotations

from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
LIB_DIR = PACKAGE_DIR / "lib"
GPU_LIB = LIB_DIR / "libksj_gpu.so"
NONCARTESIAN_PLUGIN = LIB_DIR / "libksj_gb300_noncartesian_recon.so"
COIL_COMBINE_PLUGIN = LIB_DIR / "libksj_gb300_coil_combine.so"
KB_PLUGIN = LIB_DIR / "libksj_gb300_kb_recon.so"
FIRING_HOST_LIB = LIB_DIR / "libksj_firing_host.so"


def build(verbose: bool = False):
    """Compile every native library in-tree (sm_103a)."""
    import importlib

    return importlib.import_module(__name__ + ".build").build(verbose=verbose)


class NativeLibraryMissing(RuntimeError):
    """A native library of this package is not built."""
