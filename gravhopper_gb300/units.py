"""Unit handling for the host API.

The reference works with astropy Quantities throughout and keeps kpc, km/s, Msun and
Myr internally (gravhopper/gravhopper.py:146-151).  When astropy is importable the
same Quantities are accepted and returned here.  Without astropy, plain numbers are
taken to be in those internal units (lengths kpc, velocities km/s, masses Msun,
times Myr, accelerations km/s/Myr) and plain numbers are returned.
"""
from __future__ import annotations

import numpy as np

try:  # optional, as in the reference's own optional dependencies
    from astropy import units as _u  # type: ignore
    HAVE_ASTROPY = True
except Exception:  # pragma: no cover - astropy is absent in this build's images
    _u = None
    HAVE_ASTROPY = False

# Conversion factors (see gravhopper/jbgrav.py:38-48 for the acceleration unit).
ACCEL_UNIT = 4.398600412921223e-09       # G*Msun/kpc^2 in km/s/Myr
KMS_MYR_TO_KPC = 1.022712165045695e-03   # (km/s)*Myr in kpc
G_KPC_KMS2_MSUN = 4.30091727003628e-06   # G in kpc (km/s)^2 / Msun

LENGTH, VELOCITY, MASS, TIME, ACCEL = "kpc", "km/s", "Msun", "Myr", "km/s/Myr"


def is_quantity(x) -> bool:
    return HAVE_ASTROPY and isinstance(x, _u.Quantity)


def value(x, unit: str, what: str = "value"):
    """Numeric value of ``x`` in ``unit``; plain numbers pass through unchanged."""
    if is_quantity(x):
        try:
            return x.to(_u.Unit(unit)).value
        except _u.UnitConversionError as e:
            raise ValueError(f"{what} must be convertible to {unit}.") from e
    return x


def quantity(v, unit: str):
    """Attach ``unit`` when astropy is available, else return the plain value."""
    if HAVE_ASTROPY:
        return np.asarray(v) * _u.Unit(unit)
    return v
