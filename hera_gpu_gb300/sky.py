"""Coordinate front end: equatorial -> topocentric rotations and source
directions.

The reference takes ``eq2tops`` (one 3x3 rotation per time) and ``crd_eq``
(3 x nsrc equatorial unit vectors) ready-made from its callers
(``hera_gpu/vis.py:144``); it has no builder for them.  This module derives
them from first principles so that callers (and the synthetic workloads) can
go from (LST, latitude) and (RA, Dec) to the arrays ``vis_gpu`` wants.

Conventions
-----------
Equatorial frame: x toward (RA 0h, Dec 0), y toward (RA 6h, Dec 0), z toward
the north celestial pole.  Topocentric frame: x east, y north, z up, so that
``(tx, ty)`` are the direction cosines (l, m) the beam is sampled on and
``tz > 0`` is above the horizon (the mask of ``hera_gpu/vis.py:75`` and
``tests/test_vis_gpu.py:336``).

With hour angle H = LST - RA and latitude phi, a source at (RA, Dec) has
  east  = -cos(Dec) sin(H)
  north =  cos(phi) sin(Dec) - sin(phi) cos(Dec) cos(H)
  up    =  sin(phi) sin(Dec) + cos(phi) cos(Dec) cos(H)
and expanding cos(H), sin(H) in LST and RA gives the matrix rows below.
"""
from __future__ import annotations

import numpy as np

SIDEREAL_DAY_S = 86164.0905
HERA_LATITUDE_DEG = -30.72


def eq2top(lst_rad: float, lat_rad: float) -> np.ndarray:
    """3x3 rotation taking equatorial unit vectors to topocentric (E, N, U)
    at local sidereal time ``lst_rad`` and latitude ``lat_rad``."""
    sl, cl = np.sin(lst_rad), np.cos(lst_rad)
    sp, cp = np.sin(lat_rad), np.cos(lat_rad)
    return np.array([[-sl, cl, 0.0],
                     [-sp * cl, -sp * sl, cp],
                     [cp * cl, cp * sl, sp]], dtype=np.float64)


def eq2tops(lsts_rad, lat_rad: float) -> np.ndarray:
    """Stack of :func:`eq2top` for every LST: shape (ntimes, 3, 3)."""
    return np.stack([eq2top(float(l), lat_rad) for l in np.atleast_1d(lsts_rad)])


def radec_to_crd_eq(ra_rad, dec_rad) -> np.ndarray:
    """Equatorial unit vectors for (RA, Dec) arrays: shape (3, nsrc)."""
    ra = np.asarray(ra_rad, dtype=np.float64)
    dec = np.asarray(dec_rad, dtype=np.float64)
    cd = np.cos(dec)
    return np.stack([cd * np.cos(ra), cd * np.sin(ra), np.sin(dec)])


def lst_grid(ntimes: int, hours: float = 1.0, start_rad: float = 0.0) -> np.ndarray:
    """``ntimes`` evenly spaced LSTs (radians) spanning ``hours`` of sidereal
    time from ``start_rad`` (inclusive at both ends when ntimes > 1)."""
    span = hours / 24.0 * 2 * np.pi
    if ntimes == 1:
        return np.array([start_rad])
    return start_rad + np.linspace(0.0, span, ntimes)
