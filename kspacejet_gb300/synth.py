"""Seeded synthetic MRI inputs with the shapes of the benchmark configurations.

Everything here is input generation (numpy, float64 where it matters); none
of it reconstructs anything.

* golden-angle 2-D radial trajectories in radians per pixel, (k_row, k_col),
  readout k = (n - R/2) * 2 pi / R, i.e. 2x readout oversampling relative to
  an R/2 image;
* an ellipse phantom whose continuous Fourier transform is analytic
  (ellipse -> 2 pi a b J1(kappa)/kappa with a phase ramp for its centre);
* smooth complex coil sensitivities of the form g_c * exp(i (a_c x + b_c y)),
  whose effect on k-space is an analytic shift, so multi-coil k-space of any
  size is computed exactly without a forward NUDFT;
* complex Gaussian noise at a given SNR.
"""
from __future__ import annotations

import math

import numpy as np

# pi / golden ratio = 111.246 degrees between successive spokes
GOLDEN_ANGLE = math.pi / ((1.0 + math.sqrt(5.0)) / 2.0)


def golden_angle_radial(readout: int, spokes: int, first_spoke: int = 0) -> np.ndarray:
    """[spokes * readout, 2] float32 (k_row, k_col) in radians per pixel."""
    n = np.arange(readout, dtype=np.float64)
    k = (n - readout / 2.0) * (2.0 * math.pi / readout)
    ang = (np.arange(first_spoke, first_spoke + spokes, dtype=np.float64) * GOLDEN_ANGLE) % (2.0 * math.pi)
    kr = np.outer(np.sin(ang), k)
    kc = np.outer(np.cos(ang), k)
    return np.stack([kr.ravel(), kc.ravel()], axis=-1).astype(np.float32)


def _j1_over_x(x: np.ndarray) -> np.ndarray:
    """2 J1(x) / x (= 1 at 0), from scipy when present, else a series/asymptotic mix."""
    try:
        from scipy.special import j1

        out = np.ones_like(x)
        nz = np.abs(x) > 1e-8
        out[nz] = 2.0 * j1(x[nz]) / x[nz]
        return out
    except ImportError:  # pragma: no cover
        out = np.ones_like(x)
        for i, v in np.ndenumerate(x):
            if abs(v) > 1e-8:
                out[i] = 2.0 * _j1_scalar(v) / v
        return out


def _j1_scalar(x: float) -> float:  # pragma: no cover - scipy is present on both machines
    s, term, k = 0.0, x / 2.0, 0
    while abs(term) > 1e-17 and k < 200:
        s += term
        k += 1
        term *= -(x * x / 4.0) / (k * (k + 1))
    return s


# (centre_row, centre_col, semi_row, semi_col, angle, intensity) in units of the image half-width
SHEPP_LOGAN = [
    (0.0, 0.0, 0.92, 0.69, 0.0, 1.0),
    (-0.0184, 0.0, 0.874, 0.6624, 0.0, -0.8),
    (0.0, 0.22, 0.31, 0.11, -18.0, -0.2),
    (0.0, -0.22, 0.41, 0.16, 18.0, -0.2),
    (0.35, 0.0, 0.25, 0.21, 0.0, 0.1),
    (0.1, 0.0, 0.046, 0.046, 0.0, 0.1),
    (-0.1, 0.0, 0.046, 0.046, 0.0, 0.1),
    (-0.605, -0.08, 0.046, 0.023, 0.0, 0.1),
    (-0.605, 0.0, 0.023, 0.023, 0.0, 0.1),
    (-0.605, 0.06, 0.046, 0.023, 90.0, 0.1),
]


def ellipse_kspace(traj: np.ndarray, image: int, ellipses=SHEPP_LOGAN, shift=(0.0, 0.0)) -> np.ndarray:
    """Continuous FT of an ellipse phantom sampled at `traj` ([..., 2], rad/px
    of an `image`-pixel grid), with the FT sign convention of the direct
    forward NUDFT (exp(-i k.x)), x measured in pixels from the image centre.
    `shift` moves the whole phantom (pixels)."""
    kr = traj[..., 0].astype(np.float64)
    kc = traj[..., 1].astype(np.float64)
    half = image / 2.0
    out = np.zeros(kr.shape, dtype=np.complex128)
    for (cr, cc, ar, ac, ang, rho) in ellipses:
        th = math.radians(ang)
        a, b = ar * half, ac * half
        x0, y0 = cr * half + shift[0], cc * half + shift[1]
        # rotate the frequency into the ellipse frame
        u = kr * math.cos(th) + kc * math.sin(th)
        v = -kr * math.sin(th) + kc * math.cos(th)
        kappa = np.sqrt((a * u) ** 2 + (b * v) ** 2)
        out += rho * math.pi * a * b * _j1_over_x(kappa) * np.exp(-1j * (kr * x0 + kc * y0))
    return out


def coil_parameters(channels: int, seed: int, image: int):
    """Per-coil complex gain and linear phase (rad/px) of smooth coil maps."""
    rng = np.random.default_rng(seed)
    gains = (0.5 + rng.random(channels)) * np.exp(2j * math.pi * rng.random(channels))
    slopes = rng.uniform(-3.0, 3.0, size=(channels, 2)) * (2.0 * math.pi / image)
    return gains, slopes


def multicoil_kspace(traj: np.ndarray, image: int, channels: int, seed: int, snr_db: float | None = 30.0,
                     shift=(0.0, 0.0), ellipses=SHEPP_LOGAN) -> np.ndarray:
    """[channels, M] complex64 k-space of the phantom times smooth coil maps
    g_c exp(i s_c . x) (an exact shift of the phantom's FT by s_c), plus
    complex Gaussian noise at `snr_db` relative to the mean signal power."""
    gains, slopes = coil_parameters(channels, seed, image)
    shifted = traj.astype(np.float64)[None, :, :] - slopes[:, None, :]
    out = gains[:, None] * ellipse_kspace(shifted, image, ellipses, shift)
    if snr_db is not None:
        rng = np.random.default_rng(seed + 1)
        p = np.mean(np.abs(out) ** 2)
        sigma = math.sqrt(p / (10.0 ** (snr_db / 10.0)) / 2.0)
        out += sigma * (rng.standard_normal(out.shape) + 1j * rng.standard_normal(out.shape))
    return out.astype(np.complex64)


def random_kspace(channels: int, samples: int, seed: int, frames: int | None = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    shape = (channels, samples) if frames is None else (frames, channels, samples)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def dynamic_radial(frames: int, spokes: int, readout: int, channels: int, seed: int, image: int | None = None,
                   snr_db: float | None = 30.0, motion: float = 4.0):
    """Frames of a moving ellipse: trajectory [F, spokes*readout, 2], k-space
    [F, C, spokes*readout].  Golden-angle spokes continue across frames; the
    phantom moves sinusoidally by `motion` pixels."""
    image = image if image is not None else readout // 2
    trajs, ksps = [], []
    ell = [(0.0, 0.0, 0.8, 0.6, 0.0, 1.0), (0.1, 0.1, 0.2, 0.15, 30.0, 0.5)]
    for f in range(frames):
        t = golden_angle_radial(readout, spokes, first_spoke=f * spokes)
        shift = (motion * math.sin(2 * math.pi * f / max(frames, 1)), 0.0)
        trajs.append(t)
        ksps.append(multicoil_kspace(t, image, channels, seed, snr_db, shift=shift, ellipses=ell))
    return np.stack(trajs), np.stack(ksps)


def kooshball(readout: int, spokes: int) -> np.ndarray:
    """[spokes * readout, 3] float32 (k_z, k_y, k_x) in radians per pixel: 3-D
    radial spokes through the centre along Fibonacci-sphere directions
    (z_i = 1 - (2i + 1) / spokes, azimuth i * pi (3 - sqrt 5))."""
    i = np.arange(spokes, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / spokes
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * math.pi * (3.0 - math.sqrt(5.0))
    d = np.stack([z, r * np.sin(phi), r * np.cos(phi)], axis=-1)
    k = (np.arange(readout, dtype=np.float64) - readout / 2.0) * (2.0 * math.pi / readout)
    return (d[:, None, :] * k[None, :, None]).reshape(-1, 3).astype(np.float32)
