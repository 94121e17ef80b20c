"""Seeded synthetic micro-CT data in RecView's sinogram conventions.

There is no public dataset for this path (the reference's test dataset is not available), so
benchmarks and tests use analytic phantoms:

* 2-D: random ellipses (centres uniform in a disk of radius 0.8, semi-axes U[0.05, 0.4],
  rotation U[0, pi), attenuation U[-0.2, 1.0]); lengths are in units of the field half-width
  W/2, so a line integral through the whole field is O(1).
* 3-D: random ellipsoids with the same distributions (rotation about the vertical axis); slice z
  cuts each into an ellipse.

Geometry (the reference's convention, source/general.cpp:2139-2156): image pixel (ix, iy) meets
detector sample t = (ix - h) cos(th) - (iy - h) sin(th) + c, h = W/2, c = ri->center.  With
X = ix - h and Z = h - iy that is t - c = X cos(th) + Z sin(th), the usual Radon convention.

Int16 sinograms hold round(p * LOG_SCALE) like RecView's log normalisation; raw uint16 frames
are Poisson(I0 exp(-p)) + dark with flat fields I0 = 20000 (1 + 0.02 smooth noise).
"""
from __future__ import annotations

import numpy as np

LOG_SCALE = 3000


def random_ellipses(rng: np.random.Generator, n: int) -> np.ndarray:
    """[n, 6] = (x0, z0, a, b, phi, mu) in field-half-width units."""
    r = 0.8 * np.sqrt(rng.uniform(0, 1, n))
    ang = rng.uniform(0, 2 * np.pi, n)
    x0, z0 = r * np.cos(ang), r * np.sin(ang)
    a = rng.uniform(0.05, 0.4, n)
    b = rng.uniform(0.05, 0.4, n)
    phi = rng.uniform(0, np.pi, n)
    mu = rng.uniform(-0.2, 1.0, n)
    return np.stack([x0, z0, a, b, phi, mu], axis=1)


def random_ellipsoids(rng: np.random.Generator, n: int) -> np.ndarray:
    """[n, 8] = (x0, z0, y0, a, b, c, phi, mu): y is the vertical (slice) axis."""
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    r = 0.8 * rng.uniform(0, 1, n) ** (1.0 / 3.0)
    x0, z0, y0 = (v * r[:, None]).T
    a, b, c = rng.uniform(0.05, 0.4, (3, n))
    phi = rng.uniform(0, np.pi, n)
    mu = rng.uniform(-0.2, 1.0, n)
    return np.stack([x0, z0, y0, a, b, c, phi, mu], axis=1)


def slice_heights(nslices: int) -> np.ndarray:
    """Normalised heights y of the stack's detector rows: spread over [-0.25, 0.25]."""
    return (np.arange(nslices) - (nslices - 1) / 2.0) / (max(nslices, 2) / 2.0) * 0.5


def random_spheres(rng: np.random.Generator, n: int, ixdim: int, ys: np.ndarray) -> np.ndarray:
    """[n, 5] = (x0, z0, y0, r, mu): small high-contrast spheres, radius U[1, 4] detector pixels,
    attenuation U[0.5, 2] (the ellipsoids' units), centres uniform in a disk of radius 0.8 of the
    slice plane.  Each sphere sits across one of the row heights ys (|y0 - y| < 0.9 r), so every
    sphere cuts at least one reconstructed slice."""
    half = ixdim / 2.0
    r = rng.uniform(1.0, 4.0, n) / half
    rho = 0.8 * np.sqrt(rng.uniform(0, 1, n))
    ang = rng.uniform(0, 2 * np.pi, n)
    y0 = np.asarray(ys, np.float64)[rng.integers(0, len(ys), n)] + rng.uniform(-0.9, 0.9, n) * r
    mu = rng.uniform(0.5, 2.0, n)
    return np.stack([rho * np.cos(ang), rho * np.sin(ang), y0, r, mu], axis=1)


def sphere_slice(spheres: np.ndarray, y: float) -> np.ndarray:
    """Cross-sections of spheres at height y as 2-D ellipses (discs)."""
    out = []
    for x0, z0, y0, r, mu in spheres:
        h = r * r - (y - y0) ** 2
        if h <= 0.0:
            continue
        rr = np.sqrt(h)
        out.append((x0, z0, rr, rr, 0.0, mu))
    return np.array(out, dtype=np.float64).reshape(-1, 6)


def ellipsoid_slice(ells3: np.ndarray, y: float) -> np.ndarray:
    """Cross-sections of ellipsoids at height y (normalised) as 2-D ellipses."""
    out = []
    for x0, z0, y0, a, b, c, phi, mu in ells3:
        u = (y - y0) / c
        if abs(u) >= 1.0:
            continue
        s = np.sqrt(1.0 - u * u)
        out.append((x0, z0, a * s, b * s, phi, mu))
    return np.array(out, dtype=np.float64).reshape(-1, 6)


def line_integrals(ells: np.ndarray, theta: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Analytic Radon transform p[theta, t] (FP64) of a sum of ellipses; t is the signed distance
    X cos(th) + Z sin(th) in field-half-width units."""
    th = theta[:, None]
    out = np.zeros((theta.size, t.size), dtype=np.float64)
    for x0, z0, a, b, phi, mu in ells:
        s = x0 * np.cos(th) + z0 * np.sin(th)
        d = th - phi
        a2 = (a * np.cos(d)) ** 2 + (b * np.sin(d)) ** 2
        u = t[None, :] - s
        rad = a2 - u * u
        out += np.where(rad > 0, 2.0 * mu * a * b * np.sqrt(np.maximum(rad, 0.0)) / a2, 0.0)
    return out


def detector_coords(ixdim: int, center: float) -> np.ndarray:
    """Normalised signed distance of each detector sample from the rotation centre."""
    return (np.arange(ixdim, dtype=np.float64) - center) / (ixdim / 2.0)


def angle_table(nviews: int, span_deg: float = 180.0) -> np.ndarray:
    return (np.arange(nviews, dtype=np.float64) * (span_deg / nviews)).astype(np.float32)


def sinogram_2d(seed: int, ixdim: int, nviews: int, center: float, n_ellipses: int = 10,
                noise_frac: float = 0.005) -> tuple[np.ndarray, np.ndarray]:
    """int16 log-normalised sinogram [nviews, ixdim] and the float32 angle table (degrees)."""
    rng = np.random.default_rng(seed)
    ells = random_ellipses(rng, n_ellipses)
    fdeg = angle_table(nviews)
    p = line_integrals(ells, np.deg2rad(fdeg.astype(np.float64)), detector_coords(ixdim, center))
    if noise_frac > 0:
        p = p + rng.normal(0.0, noise_frac * max(np.abs(p).max(), 1e-12), p.shape)
    sino = np.clip(np.rint(p * LOG_SCALE), -32768, 32767).astype(np.int16)
    return sino, fdeg


def smooth_noise(rng: np.random.Generator, shape: tuple[int, ...], sigma: float) -> np.ndarray:
    """Gaussian-filtered white noise with unit standard deviation (FFT convolution)."""
    w = rng.normal(size=shape)
    out = np.fft.rfftn(w)
    for ax, n in enumerate(shape):
        f = np.fft.rfftfreq(n) if ax == len(shape) - 1 else np.fft.fftfreq(n)
        g = np.exp(-2.0 * (np.pi * f * sigma) ** 2)
        sh = [1] * len(shape)
        sh[ax] = g.size
        out = out * g.reshape(sh)
    r = np.fft.irfftn(out, s=shape, axes=tuple(range(len(shape))))
    return r / max(r.std(), 1e-12)


def raw_stack(seed: int, ixdim: int, nviews: int, nslices: int, center: float,
              n_ellipsoids: int = 40, flat_level: float = 20000.0, nflat_before: int = 1,
              nflat_after: int = 1):
    """Raw uint16 frames in RecView's sinogram buffer layout.

    Returns (raw[nframes+1, nslices, ixdim] uint16 with the dark as the last frame, bInc, fdeg,
    fexp, p) where p[nslices, nviews, ixdim] are the FP64 line integrals of the SAMPLE frames.
    Frame order: flats before, samples, flats after (like docs/output*.log schedules).
    """
    rng = np.random.default_rng(seed)
    ells3 = random_ellipsoids(rng, n_ellipsoids)
    nframes = nflat_before + nviews + nflat_after
    bInc = np.zeros(nframes, dtype=np.int8)
    bInc[nflat_before:nflat_before + nviews] = 1
    fdeg = np.zeros(nframes, dtype=np.float32)
    fdeg[nflat_before:nflat_before + nviews] = angle_table(nviews)
    fexp = np.arange(nframes, dtype=np.float32)
    t = detector_coords(ixdim, center)
    theta = np.deg2rad(angle_table(nviews).astype(np.float64))
    ys = (np.arange(nslices) - (nslices - 1) / 2.0) / (max(nslices, 2) / 2.0) * 0.5
    p = np.zeros((nslices, nviews, ixdim), dtype=np.float64)
    for k, y in enumerate(ys):
        p[k] = line_integrals(ellipsoid_slice(ells3, y), theta, t)
    dark = rng.normal(100.0, 3.0, (nslices, ixdim))
    flat = flat_level * (1.0 + 0.02 * smooth_noise(rng, (nslices, ixdim), 16.0))
    raw = np.zeros((nframes + 1, nslices, ixdim), dtype=np.uint16)

    def sample(mean):
        return np.minimum(65535.0, rng.poisson(np.maximum(mean, 0.0)) + dark)

    for f in range(nframes):
        if bInc[f] & 1:
            v = f - nflat_before
            raw[f] = sample(flat * np.exp(-p[:, v, :])).astype(np.uint16)
        else:
            raw[f] = sample(flat).astype(np.uint16)
    raw[nframes] = np.clip(np.rint(dark), 0, 65535).astype(np.uint16)
    return raw, bInc, fdeg, fexp, p


def offset_ct_sinogram(seed: int, ixfrm: int, nviews360: int, nslices: int, center: float,
                       n_ellipsoids: int = 20, nflat_before: int = 1, nflat_after: int = 1,
                       noise_frac: float = 0.003):
    """Normalised int16 rows of a 360-degree offset-CT scan (rotation axis near a frame edge).

    The frame has ixfrm samples and the axis sits at `center` (frame pixels); the object fills a
    disc of radius ~ixfrm around the axis, so each frame sees one half of it and the partner frame
    180 degrees later the other.  Returns (sino[nframes+1, nslices, ixfrm] int16 with a zero dark
    frame last, bInc, fdeg) with flats before and after the samples, angles 360 v / nviews360.
    """
    rng = np.random.default_rng(seed)
    ells3 = random_ellipsoids(rng, n_ellipsoids)
    ns = nviews360 + 1
    nframes = nflat_before + ns + nflat_after
    bInc = np.zeros(nframes, dtype=np.int8)
    bInc[nflat_before:nflat_before + ns] = 1
    fdeg = np.zeros(nframes, dtype=np.float32)
    ang = (np.arange(ns, dtype=np.float64) * (360.0 / nviews360)).astype(np.float32)
    fdeg[nflat_before:nflat_before + ns] = ang
    fdeg[nflat_before + ns:] = 360.0
    # field half-width = ixfrm: the stitched row is twice the frame
    t = (np.arange(ixfrm, dtype=np.float64) - center) / float(ixfrm)
    theta = np.deg2rad(ang.astype(np.float64))
    ys = (np.arange(nslices) - (nslices - 1) / 2.0) / (max(nslices, 2) / 2.0) * 0.5
    sino = np.zeros((nframes + 1, nslices, ixfrm), dtype=np.int16)
    for k, y in enumerate(ys):
        p = line_integrals(ellipsoid_slice(ells3, y), theta, t)
        if noise_frac > 0:
            p = p + rng.normal(0.0, noise_frac * max(np.abs(p).max(), 1e-12), p.shape)
        sino[nflat_before:nflat_before + ns, k] = np.clip(np.rint(p * LOG_SCALE), -32768, 32767)
    return sino, bInc, fdeg
