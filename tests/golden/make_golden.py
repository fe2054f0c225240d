"""Generate the golden fixtures under tests/golden/ from the KSpaceJet
reference itself.

Run in a tree where the reference sources exist (it builds them with
oracle/build.py into oracle/_ref/ and calls them through oracle.Reference):

    python tests/golden/make_golden.py [--reference-root PATH]

Every input below is either copied from a reference unit test (file:line
given) or drawn from a fixed seed; every expected output is what the
compiled reference returns for it.  The fixtures travel with the repository,
so machines without the reference tree still check against them.
"""
from __future__ import annotations

import argparse
import json
import math
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import build as obuild  # noqa: E402

PI32 = np.float32(math.pi)


def radial_spokes(nro: int, spokes: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0.0, math.pi, spokes)
    k = (np.arange(nro) - nro / 2.0) * (2.0 * math.pi / nro)
    return np.stack([np.outer(np.sin(ang), k).ravel(), np.outer(np.cos(ang), k).ravel()], -1).astype(np.float32)


def cplx(rng, *shape, dtype=np.complex64):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def type_digests(reference_root: Path) -> dict:
    h = (reference_root / "libs/recon/kspacejet-provider-sdk/include/kspacejet/provider/type_registry.h").read_text()
    out = {}
    for name in ["noncartesian_kspace_frame", "trajectory_frame", "coil_image_frame", "image_frame"]:
        i = h.index(f"ksj_type_registry_{name}_identity_digest =")
        out[name] = "".join(re.findall(r"UINT8_C\(0x([0-9a-f]{2})\)", h[i:i + 2000])[:32])
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=str(obuild.DEFAULT_REFERENCE_ROOT))
    args = ap.parse_args()
    root = Path(args.reference_root)
    if not obuild.build_reference(root):
        print("reference tree not found; fixtures unchanged", file=sys.stderr)
        return 1
    ref = oracle.Reference()
    fx: dict[str, np.ndarray] = {}

    # radial_gridding_tests.cpp:16-29 -- analytic ramp known answers
    t = np.array([[0.0, 0.0], [3.0 / 5.0, 4.0 / 5.0], [-math.pi, 0.0]])
    fx["ramp_traj"] = t
    fx["ramp_out"] = ref.ramp_dcf(t)

    # radial_gridding_tests.cpp:92-125 -- one off-bin sample splits 1, 1, 0, 0
    s = np.array([2.0 / math.pi + 0j])
    tr = np.array([[math.pi / 2.0, 0.0]])
    fx["offbin_samples"], fx["offbin_traj"] = s, tr
    fx["offbin_out"] = ref.linear_gridding(2, 2, s, tr, ref.ramp_dcf(tr), 0.0, 0.0)

    # radial_gridding_tests.cpp:31-90 -- Cartesian-bin spokes == weighted direct NUDFT (4x4, origin (1.5, 0.5))
    s = np.array([1.0 - 0.5j, -2.0 + 0.25j, 0.5 + 3.0j, 1.5 - 1.0j, -0.75 - 0.25j])
    tr = np.array([[-math.pi / 2, 0.0], [0.0, 0.0], [math.pi / 2, 0.0], [0.0, -math.pi / 2], [0.0, math.pi / 2]])
    d = ref.ramp_dcf(tr)
    fx["cartbin_samples"], fx["cartbin_traj"] = s, tr
    fx["cartbin_out"] = ref.linear_gridding(4, 4, s, tr, d, 1.5, 0.5)
    fx["cartbin_direct"] = ref.direct_adjoint(4, 4, s * d, tr, 1.5, 0.5)

    # radial_gridding_tests.cpp:127-165 -- the 3x4 byte-identity fixture (float)
    s = np.array([0.5 + 1.0j, -1.0 + 0.25j, 2.0 - 0.75j], dtype=np.complex64)
    tr = np.array([[-PI32 / np.float32(3), 0], [0, PI32 / np.float32(2)], [PI32 / np.float32(4), -PI32 / np.float32(3)]],
                  dtype=np.float32)
    fx["repeat_samples"], fx["repeat_traj"] = s, tr
    fx["repeat_out"] = ref.linear_gridding(3, 4, s, tr, ref.ramp_dcf(tr), 0.0, 0.0)

    # noncartesian_recon_provider_tests.cpp:71-78 -- the HostState payloads
    k = np.array([1 + 2j, 3 - 1j, 10 - 4j, -2 + 7j], dtype=np.complex64)
    tr = np.array([[0.0, 0.0], [PI32, -np.float32(0.5) * PI32]], dtype=np.float32)
    fx["host_kspace"], fx["host_traj"] = k, tr
    fx["host_radial_1ch"] = ref.linear_gridding(2, 2, k[:2], tr, ref.ramp_dcf(tr), 0.5, 0.5)
    fx["host_direct_ch0"] = ref.direct_adjoint(2, 2, k[:2], tr, 0.5, 0.5)
    fx["host_direct_ch1"] = ref.direct_adjoint(2, 2, k[2:], tr, 0.5, 0.5)

    # radial_rss_hdf5_tests.cpp:187-232 -- 2x4 rectangular radial, origin (0.5, 1.5), two coils, RSS
    tr = np.array([[PI32 / np.float32(2), PI32 / np.float32(4)], [PI32 / np.float32(4), -PI32 / np.float32(2)]],
                  dtype=np.float32)
    c0 = np.array([1 + 0j, 2 + 0j], dtype=np.complex64)
    c1 = np.array([3 + 0j, 4 + 0j], dtype=np.complex64)
    dd = ref.ramp_dcf(tr)
    i0 = ref.linear_gridding(2, 4, c0, tr, dd, 0.5, 1.5)
    i1 = ref.linear_gridding(2, 4, c1, tr, dd, 0.5, 1.5)
    fx["rect_traj"], fx["rect_coils"] = tr, np.stack([c0, c1])
    fx["rect_images"] = np.stack([i0, i1])
    fx["rect_rss"] = np.sqrt(np.abs(i0) ** 2 + np.abs(i1) ** 2).astype(np.float32)

    # coil_combine_provider_tests.cpp:61-70, 299-320 -- RSS 5, 12, 13, sqrt(6)
    fx["rss_input"] = np.array([3 + 4j, 0, 0, 12j, 5, 12j, 1 + 1j, 2j], dtype=np.complex64).reshape(2, 2, 2)
    fx["rss_out"] = np.array([5.0, 12.0, 13.0, math.sqrt(6.0)], dtype=np.float32).reshape(2, 2)

    # nufft_tests.cpp:12-32, 50-68 -- direct adjoint of a k=0 sample fills every pixel
    fx["dc_out"] = ref.direct_adjoint(2, 3, np.array([2.0 - 1.0j]), np.array([[0.0, 0.0]]), 0.5, 1.0)

    # seeded multi-coil cases through the reference's float and double overloads
    for name, (n, nro, spokes, ch, seed) in {"med32": (32, 64, 9, 3, 11), "med64": (64, 128, 13, 2, 12),
                                              "smallrect": (16, 32, 5, 2, 13)}.items():
        rng = np.random.default_rng(seed)
        tr = radial_spokes(nro, spokes, seed)
        m = tr.shape[0]
        ks = cplx(rng, ch, m)
        d32 = ref.ramp_dcf(tr)
        d64 = ref.ramp_dcf(tr.astype(np.float64))
        rows, cols = (n, n) if name != "smallrect" else (n // 2, n)
        f32 = np.stack([ref.linear_gridding(rows, cols, ks[c], tr, d32) for c in range(ch)])
        f64 = np.stack([ref.linear_gridding(rows, cols, ks[c].astype(np.complex128), tr.astype(np.float64), d64)
                        for c in range(ch)])
        fx[f"{name}_traj"], fx[f"{name}_kspace"] = tr, ks
        fx[f"{name}_shape"] = np.array([rows, cols])
        fx[f"{name}_ref_f32"], fx[f"{name}_ref_f64"] = f32, f64

    np.savez_compressed(HERE / "reference_fixtures.npz", **fx)
    (HERE / "type_registry.json").write_text(json.dumps(type_digests(root), indent=1, sort_keys=True) + "\n")
    print("wrote", HERE / "reference_fixtures.npz", "and", HERE / "type_registry.json")
    return 0


if __name__ == "__main__":
    sys.exit(main())
