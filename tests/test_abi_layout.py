"""The restated Provider ABI is the reference's, byte for byte; the payload
type table equals the reference registry; the native libraries export what
the headers declare."""
import ctypes
import json
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF_HEADER_DIR = Path("/root/reference/libs/recon/kspacejet-provider-sdk/include")


def _probe(tmp_path, header: Path, incdir: Path) -> str:
    exe = tmp_path / f"probe_{abs(hash(str(header)))}"
    subprocess.run(["gcc", "-std=c11", f'-DKSJ_ABI_HEADER="{header}"', "-I", str(incdir),
                    str(ROOT / "tests/abi_layout_probe.c"), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_probe_runs_on_restated_header(tmp_path):
    out = _probe(tmp_path, ROOT / "include/ksj_provider_abi.h", ROOT / "include")
    assert "ksj_provider_api 112" in out  # 32-byte header + 10 pointers
    assert "ksj_type_descriptor_view" in out


@pytest.mark.skipif(not REF_HEADER_DIR.exists(), reason="reference tree not present on this machine")
def test_layout_identical_to_reference_header(tmp_path):
    mine = _probe(tmp_path, ROOT / "include/ksj_provider_abi.h", ROOT / "include")
    ref = _probe(tmp_path, REF_HEADER_DIR / "kspacejet/provider/provider.h", REF_HEADER_DIR)
    assert mine == ref


def test_type_table_matches_reference_registry():
    table = (ROOT / "kspacejet_gb300/csrc/provider/abi_support.hpp").read_text()
    golden = json.loads((ROOT / "tests/golden/type_registry.json").read_text())
    for name, digest in golden.items():
        assert digest in table, name


def _declared(header: Path, prefix: str) -> list[str]:
    text = header.read_text()
    return sorted(set(re.findall(rf"\b({prefix}\w+)\s*\(", text)) - {prefix})


def test_gpu_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(str(native.GPU_LIB))
    names = _declared(ROOT / "include/ksj_gpu.h", "ksj_gpu_") + _declared(ROOT / "include/ksj_gpu.h", "ksj_coil_")
    names += _declared(ROOT / "include/ksj_serve.h", "ksj_serve_")
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n


def test_plugins_export_exactly_the_query_symbol(native):
    for path in (native.NONCARTESIAN_PLUGIN, native.COIL_COMBINE_PLUGIN):
        out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True).stdout
        syms = {line.split()[-1] for line in out.splitlines() if " T " in line}
        assert syms == {"ksj_provider_query"}, syms
