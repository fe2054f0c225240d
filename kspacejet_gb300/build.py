"""In-tree build of the native libraries (no CMake; a few translation units
compiled in parallel).

* ``lib/libksj_gpu.so``      -- the sm_103a kernels behind ``include/ksj_gpu.h``
* ``lib/libksj_gb300_noncartesian_recon.so`` -- drop-in ``org.kspacejet.noncartesian-recon`` plug-in
* ``lib/libksj_gb300_coil_combine.so``       -- drop-in ``org.kspacejet.coil-combine`` plug-in
* ``lib/libksj_gb300_kb_recon.so``           -- ``org.kspacejet.gb300-noncartesian-recon`` (Kaiser-Bessel operators)
* ``lib/libksj_firing_host.so``              -- synchronous Provider host used by tests and the bench

Every CUDA unit is compiled for ``-gencode arch=compute_103a,code=sm_103a``
only.  Outputs are written atomically and rebuilt when a source is newer.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OBJ = PKG / "_build"
LIB = PKG / "lib"

GPU_LIB = LIB / "libksj_gpu.so"
NONCARTESIAN_PLUGIN = LIB / "libksj_gb300_noncartesian_recon.so"
COIL_COMBINE_PLUGIN = LIB / "libksj_gb300_coil_combine.so"
KB_PLUGIN = LIB / "libksj_gb300_kb_recon.so"
FIRING_HOST = LIB / "libksj_firing_host.so"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                     "-I" + str(INCLUDE), "-I" + str(CSRC)]
CXX_FLAGS = ["-std=c++20", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wno-unused-const-variable",
             "-I" + str(INCLUDE)]

CU_SOURCES = ["ksj_gpu_gridding.cu", "ksj_gpu_misc.cu", "ksj_gpu_combine.cu", "ksj_gpu_forward.cu", "ksj_serve.cu"]
GPU_HEADERS = [CSRC / "ksj_gpu_internal.cuh", INCLUDE / "ksj_gpu.h", INCLUDE / "ksj_serve.h"]
PLUGIN_HEADERS = [CSRC / "provider/abi_support.hpp", INCLUDE / "ksj_provider_abi.h", INCLUDE / "ksj_gpu.h"]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout[-3000:]}"
                           f"\n{proc.stderr[-6000:]}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _tmp(p: Path) -> Path:
    return p.with_name(p.name + f".tmp{os.getpid()}")


def _compile_cu(name: str) -> Path:
    src = CSRC / name
    obj = OBJ / (Path(name).stem + ".o")
    if _stale(obj, [src, Path(__file__)] + GPU_HEADERS):
        tmp = _tmp(obj)
        _run([NVCC] + NVCC_FLAGS + ["-c", str(src), "-o", str(tmp)])
        os.replace(tmp, obj)
    return obj


def _link_gpu(objs: list[Path]) -> None:
    if _stale(GPU_LIB, objs):
        tmp = _tmp(GPU_LIB)
        _run([NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", str(tmp)] + [str(o) for o in objs])
        os.replace(tmp, GPU_LIB)


def _plugin(src: Path, out: Path) -> None:
    if _stale(out, [src, GPU_LIB, Path(__file__)] + PLUGIN_HEADERS):
        tmp = _tmp(out)
        _run(["g++"] + CXX_FLAGS + ["-shared", "-DKSJ_PROVIDER_BUILDING_PLUGIN=1", str(src), "-o", str(tmp),
                                    "-L" + str(LIB), "-l:libksj_gpu.so", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, out)


def _host() -> None:
    src = CSRC / "host/firing_host.cpp"
    if _stale(FIRING_HOST, [src, Path(__file__)] + PLUGIN_HEADERS):
        tmp = _tmp(FIRING_HOST)
        _run(["g++"] + CXX_FLAGS + ["-shared", str(src), "-o", str(tmp), "-ldl"])
        os.replace(tmp, FIRING_HOST)


def build(verbose: bool = False) -> list[Path]:
    OBJ.mkdir(parents=True, exist_ok=True)
    LIB.mkdir(parents=True, exist_ok=True)
    with ThreadPoolExecutor(max_workers=4) as pool:
        host = pool.submit(_host)
        objs = list(pool.map(_compile_cu, CU_SOURCES))
        _link_gpu(objs)
        plugins = [pool.submit(_plugin, CSRC / "provider/noncartesian_recon_provider.cpp", NONCARTESIAN_PLUGIN),
                   pool.submit(_plugin, CSRC / "provider/coil_combine_provider.cpp", COIL_COMBINE_PLUGIN),
                   pool.submit(_plugin, CSRC / "provider/kb_recon_provider.cpp", KB_PLUGIN)]
        for f in plugins + [host]:
            f.result()
    out = [GPU_LIB, NONCARTESIAN_PLUGIN, COIL_COMBINE_PLUGIN, KB_PLUGIN, FIRING_HOST]
    if verbose:
        for p in out:
            print(p)
    return out


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
