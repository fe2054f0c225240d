"""Build recipe for the parity checker (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``ksj_oracle.c`` into
  ``oracle/_build/libksj_oracle.so``.  It needs only gcc and runs on every host.
* ``build_reference()`` compiles the KSpaceJet reference's own sources, where
  they lie, into ``oracle/_ref/``:

  - ``libksj_ref.so``: the reference's radial-gridding / direct-NUDFT numerics
    (``libs/numerics/kspacejet-nufft/src/...``) behind the C wrappers of
    ``ref_shim.cpp``;
  - ``libref_noncartesian_recon.so``: the reference's own
    ``org.kspacejet.noncartesian-recon`` Provider plug-in, built from its
    sources, so the host harness can drive the reference and the CUDA Provider
    through the same C ABI.

  The reference tree is only read, never written; its CMake build is not used
  (it needs Conan packages absent here).  The one missing dependency on this
  path, the spdlog-backed logging header, is replaced by
  ``oracle/ref_include/kspacejet/logging/logging.hpp``.  The reference's
  coil-combine Provider is not built: its RSS lives in an Eigen translation
  unit and Eigen is not installed, so RSS parity rests on the restatement and
  the reference tests' known answers.

Both builds use ``-std=c++20`` / ``-ffp-contract=off`` (the reference's CMake
sets ``CMAKE_CXX_EXTENSIONS OFF``, under which GCC does not contract a*b+c).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"
DEFAULT_REFERENCE_ROOT = Path("/root/reference")

ORACLE_LIB = BUILD_DIR / "libksj_oracle.so"
REF_NUMERICS_LIB = REF_DIR / "libksj_ref.so"
REF_PROVIDER_LIB = REF_DIR / "libref_noncartesian_recon.so"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stderr[-4000:]}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement.  Returns the shared-library path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    src = HERE / "ksj_oracle.c"
    if force or _stale(ORACLE_LIB, [src, Path(__file__)]):
        tmp = ORACLE_LIB.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fvisibility=hidden",
              str(src), "-o", str(tmp), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def _reference_includes(root: Path) -> list[str]:
    incs = ["-I" + str(HERE / "ref_include")]
    for d in sorted((root / "libs").rglob("include")):
        if d.is_dir():
            incs.append("-I" + str(d))
    return incs


def build_reference(reference_root: Path | str | None = None, force: bool = False) -> bool:
    """Compile the reference's numerics and radial Provider from its own
    sources.  Returns False (and builds nothing) when the reference tree is
    absent, as on a machine that only carries this repository."""
    root = Path(reference_root) if reference_root else DEFAULT_REFERENCE_ROOT
    nufft = root / "libs/numerics/kspacejet-nufft/src"
    if not nufft.is_dir():
        return False
    REF_DIR.mkdir(parents=True, exist_ok=True)
    cxx = ["g++", "-std=c++20", "-O3", "-fPIC", "-shared", "-ffp-contract=off"]
    incs = _reference_includes(root)
    numerics_srcs = [nufft / "eigen/eigen_radial_gridding.cpp", nufft / "eigen/eigen_nufft_direct_nudft.cpp",
                     nufft / "nufft.cpp", nufft / "bart/bart_nufft2.cpp"]
    memory_srcs = sorted((root / "libs/core/kspacejet-memory/src").glob("*.cpp"))
    shim = HERE / "ref_shim.cpp"
    if force or _stale(REF_NUMERICS_LIB, numerics_srcs + [shim]):
        tmp = REF_NUMERICS_LIB.with_suffix(f".so.tmp{os.getpid()}")
        _run(cxx + ["-fvisibility=hidden"] + incs + [str(s) for s in [shim] + numerics_srcs + memory_srcs]
             + ["-o", str(tmp)])
        os.replace(tmp, REF_NUMERICS_LIB)
    prov = root / "providers/kspacejet-noncartesian-recon/src"
    prov_srcs = [prov / "provider_entry.cpp", prov / "provider_api.cpp"] + sorted((prov / "operators").glob("*.cpp"))
    if force or _stale(REF_PROVIDER_LIB, prov_srcs + numerics_srcs):
        tmp = REF_PROVIDER_LIB.with_suffix(f".so.tmp{os.getpid()}")
        _run(cxx + ["-fvisibility=hidden", "-DKSJ_PROVIDER_BUILDING_PLUGIN=1"] + incs + ["-I" + str(prov)]
             + [str(s) for s in prov_srcs + numerics_srcs + memory_srcs] + ["-o", str(tmp)])
        os.replace(tmp, REF_PROVIDER_LIB)
    return True


def main(argv: list[str]) -> int:
    force = "--force" in argv
    print("oracle:", build_oracle(force=force))
    print("reference built:", build_reference(force=force))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
