"""Comparison helpers shared by the tests."""
from __future__ import annotations

import numpy as np


def site_rel_err(out, ref, scale):
    """max_i |out_i - ref_i| / max(|ref_i|, scale_i): a per-site relative error whose
    denominator does not vanish where the result cancels.  scale_i is the magnitude of the
    terms that were summed at site i (e.g. 1/2 sum |U||psi| + m|psi|)."""
    den = np.maximum(np.abs(ref), scale)
    den = np.where(den == 0, 1.0, den)
    return float(np.max(np.abs(out - ref) / den))


def staggered_scale(U, psi, mass, lx, ly):
    """Per-site sum of the magnitudes of the terms of D psi (operators.cpp:207-238)."""
    P = psi.reshape(ly, lx)
    a = np.abs(P)
    Ux = np.abs(U[0::2]).reshape(ly, lx)
    Uy = np.abs(U[1::2]).reshape(ly, lx)
    s = (Ux * np.roll(a, -1, 1) + np.roll(Ux, 1, 1) * np.roll(a, 1, 1) +
         Uy * np.roll(a, -1, 0) + np.roll(Uy, 1, 0) * np.roll(a, 1, 0))
    return (0.5 * s + abs(mass) * a).reshape(-1)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
