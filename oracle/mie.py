"""Mie series of a dielectric circular cylinder: the known-answer far field
and near-field ring.

TEST INFRASTRUCTURE (the oracle's physics check).  The CW path of the
reference (scatteredWave, mpiTM_UPML.c:337-374 / mpiTE_UPML.c:250-281, and
the frequency-domain NTFF, ntffTM.c:72-158 / ntffTE.c:242-338) computes the
field scattered by a cylinder of radius a and refractive index m under a unit
plane wave exp(i(k x.d - w t)), d = (cos t_in, sin t_in).  In two dimensions
the exact answer is the published series (Bohren & Huffman, "Absorption and
Scattering of Light by Small Particles", section 8.4):

  outside: E_sc = sum_n i^n b_n H_n(k r) exp(i n (phi - t_in))
  far field: E_sc ~ sqrt(2 / (pi k r)) exp(i (k r - pi/4)) T(phi),
             T(phi) = sum_n b_n exp(i n (phi - t_in))

with, from continuity of the axial field and of its normal derivative
(weighted by 1/eps for the H-polarised case),

  b_n = (q J_n'(m x) J_n(x) - J_n'(x) J_n(m x)) / (H_n'(x) J_n(m x) - q J_n'(m x) H_n(x))

x = k a, q = m for E polarisation (TM here: Ez, Hx, Hy) and q = 1/m for H
polarisation (TE here: Ex, Ey, Hz).  H_n is the Hankel function of the first
kind; b_{-n} = b_n.
"""
from __future__ import annotations

import numpy as np


def coefficients(x: float, m: float, pol: str, nmax: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """(n, b_n) for n = -nmax..nmax; nmax defaults to the Wiscombe-type bound
    x + 4 x^(1/3) + 10 (enough for |b_n| to fall below double rounding)."""
    from scipy.special import h1vp, hankel1, jv, jvp
    if pol not in ("TM", "TE"):
        raise ValueError("pol is 'TM' (E along the axis) or 'TE' (H along the axis)")
    if nmax is None:
        nmax = int(np.ceil(x + 4.0 * x ** (1.0 / 3.0) + 10))
    n = np.arange(-nmax, nmax + 1)
    mx = m * x
    J, Jp = jv(n, x), jvp(n, x)
    Jm, Jmp = jv(n, mx), jvp(n, mx)
    H, Hp = hankel1(n, x), h1vp(n, x)
    q = m if pol == "TM" else 1.0 / m
    b = (q * Jmp * J - Jp * Jm) / (Hp * Jm - q * Jmp * H)
    return n, b


def far_field(radius: float, wavelength: float, eps: float, pol: str, incidence_deg: float = 0.0,
              angles_deg=None) -> np.ndarray:
    """T(phi) at the given observation angles (default 0..359 degrees, the
    NTFF's 360 directions); radius and wavelength in the same unit."""
    if angles_deg is None:
        angles_deg = np.arange(360)
    phi = np.deg2rad(np.asarray(angles_deg, dtype=float))
    x = 2.0 * np.pi * radius / wavelength
    n, b = coefficients(x, float(np.sqrt(eps)), pol)
    t_in = np.deg2rad(incidence_deg)
    return np.exp(1j * np.outer(phi - t_in, n)) @ b


def pattern_error(intensity: np.ndarray, reference: np.ndarray) -> tuple[float, float]:
    """(relative L2 error, scale) of an intensity pattern against a reference
    pattern after the least-squares scale s: |I - s R| / |I|.  The scale
    absorbs the solvers' own far-field normalisation (R0, h_u factors)."""
    intensity = np.asarray(intensity, dtype=float)
    reference = np.asarray(reference, dtype=float)
    s = float(intensity @ reference / (reference @ reference))
    return float(np.linalg.norm(intensity - s * reference) / np.linalg.norm(intensity)), s


def near_field_ring(radius: float, wavelength: float, eps: float, pol: str, ring_radius: float,
                    angles_deg=None) -> np.ndarray:
    """|E|^2 of the scattered field on a circle about the cylinder's axis
    (same length unit throughout): the axial E_z (TM) or, for H polarisation
    with the plane wave along +x, E_y obtained from H_z = sum i^n b_n H_n(kr)
    e^{in phi} through E_y ~ (1/k) dH_z/dx (unit incident E_y):

      TM: |sum_n i^n b_n H_n(kr) e^{in phi}|^2
      TE: |sum_n i^n b_n (cos(phi) H_n'(kr) - i n sin(phi) H_n(kr) / (kr)) e^{in phi}|^2

    The default angles are those of field_outputElliptic's ring (field.c:322-343),
    180 down to 0 degrees, i.e. entry q is the angle 180 - q."""
    from scipy.special import h1vp, hankel1
    if angles_deg is None:
        angles_deg = np.arange(180, -1, -1)
    phi = np.deg2rad(np.asarray(angles_deg, dtype=float))[:, None]
    n, b = coefficients(2.0 * np.pi * radius / wavelength, float(np.sqrt(eps)), pol)
    kr = 2.0 * np.pi * ring_radius / wavelength
    H = hankel1(n, kr)[None, :]
    w = ((1j ** n) * b)[None, :] * np.exp(1j * phi * n[None, :])
    if pol == "TM":
        return np.abs((w * H).sum(axis=1)) ** 2
    Hp = h1vp(n, kr)[None, :]
    return np.abs((w * (np.cos(phi) * Hp - 1j * n[None, :] * np.sin(phi) / kr * H)).sum(axis=1)) ** 2
