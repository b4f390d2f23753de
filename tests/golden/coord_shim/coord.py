"""A test-only stand-in for the parts of the `coord` package (LSSTDESC.Coord, a dependency of
TreeCorr's Python layer that this image does not have) which TreeCorr's correlation path
uses: AngleUnit (its valid names, lookup by name and value in radians), the unit constants,
Angle (a value in radians with unit arithmetic) and CelestialCoord (ra, dec and the unit
vector).  Written from the package's documented interface for tests/golden/make_api_trace.py,
which runs TreeCorr's own Python on top of the reference's compiled module to record the
calls it makes across the `_treecorr` boundary.  It is not the package, and nothing outside
that script imports it.
"""
import math


class AngleUnit:
    """A unit of angle: value = the size of one unit in radians."""

    valid_names = ['rad', 'deg', 'hr', 'hour', 'arcmin', 'arcsec']
    _values = {'rad': 1.0, 'deg': math.pi / 180.0, 'hr': math.pi / 12.0,
               'hour': math.pi / 12.0, 'arcmin': math.pi / 180.0 / 60.0,
               'arcsec': math.pi / 180.0 / 3600.0}

    def __init__(self, value):
        self.value = float(value)

    @classmethod
    def from_name(cls, name):
        """The unit whose name the given string starts with ('degrees' -> deg)."""
        s = name.strip().lower()
        for n in sorted(cls.valid_names, key=len, reverse=True):
            if s.startswith(n):
                return cls(cls._values[n])
        raise ValueError("Unknown angle unit: %s" % name)

    def __rmul__(self, x):
        return Angle(x, self)

    def __eq__(self, other):
        return isinstance(other, AngleUnit) and self.value == other.value

    def __hash__(self):
        return hash(self.value)

    def __repr__(self):
        return "coord.AngleUnit(%r)" % self.value


radians = AngleUnit(1.0)
degrees = AngleUnit(math.pi / 180.0)
hours = AngleUnit(math.pi / 12.0)
arcmin = AngleUnit(math.pi / 180.0 / 60.0)
arcsec = AngleUnit(math.pi / 180.0 / 3600.0)


class Angle:
    """An angle, stored in radians."""

    def __init__(self, theta, unit=None):
        if isinstance(theta, Angle):
            self._rad = theta._rad
        else:
            self._rad = float(theta) * (unit.value if unit is not None else 1.0)

    @property
    def rad(self):
        return self._rad

    @property
    def deg(self):
        return self._rad / degrees.value

    def __truediv__(self, other):
        if isinstance(other, AngleUnit):
            return self._rad / other.value
        return Angle(self._rad / other)

    def __mul__(self, x):
        return Angle(self._rad * x)

    __rmul__ = __mul__

    def __float__(self):
        return self._rad

    def __repr__(self):
        return "coord.Angle(%r, coord.radians)" % self._rad


class CelestialCoord:
    """A position on the sphere (ra, dec)."""

    def __init__(self, ra, dec):
        self.ra = ra if isinstance(ra, Angle) else Angle(ra)
        self.dec = dec if isinstance(dec, Angle) else Angle(dec)

    def get_xyz(self):
        cd = math.cos(self.dec.rad)
        return (cd * math.cos(self.ra.rad), cd * math.sin(self.ra.rad), math.sin(self.dec.rad))
