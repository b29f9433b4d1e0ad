"""Milling cutters, mirroring the reference's cutter classes and constructors.

Each class builds the flat CutterDesc that crosses the C ABI.  Derived
quantities (radius, center height, composite radius/height/z-offset tables)
are computed by the native code from these constructor arguments exactly as
the reference constructors do; the composite presets below restate
src/cutters/compositecutter.cpp:296-383 so that e.g. BallConeCutter(2, 6, pi/4)
carries the same sub-cutters, radius windows and z offsets.
"""
from __future__ import annotations

import math

from . import _abi


class MillingCutter:
    """Base class (src/cutters/millingcutter.hpp:50-196)."""

    kind = 0

    def desc(self) -> _abi.CutterDesc:
        raise NotImplementedError

    def getRadius(self) -> float:
        return self.radius

    def getDiameter(self) -> float:
        return self.diameter

    def getLength(self) -> float:
        return self.length

    def _sub(self) -> _abi.SubCutter:
        s = _abi.SubCutter()
        s.kind = self.kind
        s.diameter = self.diameter
        s.corner_radius = getattr(self, "corner_radius", 0.0)
        s.angle = getattr(self, "angle", 0.0)
        s.length = self.length_arg
        return s

    def __repr__(self):
        return self.str()


class _Basic(MillingCutter):
    def desc(self) -> _abi.CutterDesc:
        d = _abi.CutterDesc()
        d.kind = self.kind
        d.nsub = 0
        d.base = self._sub()
        return d


class CylCutter(_Basic):
    """CylCutter(d, l) (src/cutters/cylcutter.cpp:39-46)."""

    kind = _abi.CUTTER_CYL

    def __init__(self, d: float, l: float):
        if not (d > 0.0 and l > 0.0):
            raise ValueError("CylCutter needs d > 0 and l > 0")
        self.diameter = float(d)
        self.radius = d / 2.0
        self.length = float(l)
        self.length_arg = float(l)

    def str(self):
        return f"CylCutter (d={self.diameter}, L={self.length})"


class BallCutter(_Basic):
    """BallCutter(d, l) (src/cutters/ballcutter.cpp:38-45)."""

    kind = _abi.CUTTER_BALL

    def __init__(self, d: float, l: float):
        if not (d > 0.0 and l > 0.0):
            raise ValueError("BallCutter needs d > 0 and l > 0")
        self.diameter = float(d)
        self.radius = d / 2.0
        self.length = float(l)
        self.length_arg = float(l)

    def str(self):
        return f"BallCutter(d={self.diameter}, r={self.radius}, L={self.length})"


class BullCutter(_Basic):
    """BullCutter(d, r, l) (src/cutters/bullcutter.cpp:38-47)."""

    kind = _abi.CUTTER_BULL

    def __init__(self, d: float, r: float, l: float):
        if not (d > 0.0 and l > 0.0 and d / 2.0 - r > 0.0 and r > 0.0):
            raise ValueError("BullCutter needs d > 0, 0 < r < d/2 and l > 0")
        self.diameter = float(d)
        self.radius = d / 2.0
        self.corner_radius = float(r)
        self.length = float(l)
        self.length_arg = float(l)

    def str(self):
        return f"BullCutter(d={self.diameter}, r1={self.radius - self.corner_radius} r2={self.corner_radius}, L={self.length})"


class ConeCutter(_Basic):
    """ConeCutter(d, angle, l=10) (src/cutters/conecutter.cpp:39-49); angle is
    the half-angle in radians."""

    kind = _abi.CUTTER_CONE

    def __init__(self, d: float, angle: float, l: float = 10.0):
        if not (angle > 0.0 and d > 0.0):
            raise ValueError("ConeCutter needs d > 0 and angle > 0")
        self.diameter = float(d)
        self.radius = d / 2.0
        self.angle = float(angle)
        self.length_arg = float(l)
        self.length = self.radius / math.tan(self.angle) + l
        self.center_height = self.radius / math.tan(self.angle)

    def str(self):
        return f"ConeCutter (d={self.diameter}, angle={self.angle}, L={self.length})"


class CompositeCutter(MillingCutter):
    """CompositeCutter (src/cutters/compositecutter.cpp:35-51): sub-cutter n
    applies from radiusvec[n-1] to radiusvec[n], shifted by zoffset[n]."""

    kind = _abi.CUTTER_COMPOSITE

    def __init__(self):
        self.parts = []
        self.radius = 0.0
        self.diameter = 0.0
        self.length = 0.0

    def addCutter(self, c: MillingCutter, r: float, h: float, zoff: float):
        if isinstance(c, CompositeCutter):
            raise TypeError("nested CompositeCutter is not supported")
        if len(self.parts) >= _abi.MAX_SUB:
            raise ValueError(f"at most {_abi.MAX_SUB} sub-cutters")
        self.parts.append((c, float(r), float(h), float(zoff)))
        if r > self.radius:
            self.radius = float(r)
            self.diameter = 2 * r

    def desc(self) -> _abi.CutterDesc:
        d = _abi.CutterDesc()
        d.kind = _abi.CUTTER_COMPOSITE
        d.nsub = len(self.parts)
        for n, (c, r, h, z) in enumerate(self.parts):
            s = c._sub()
            s.radius = r
            s.height = h
            s.zoffset = z
            d.sub[n] = s
        d.composite_length = self.length
        return d

    def str(self):
        return f"CompositeCutter with {len(self.parts)} cutters"


class CompCylCutter(CompositeCutter):
    def __init__(self, diam2: float, clength: float):
        super().__init__()
        self.addCutter(CylCutter(diam2, clength), diam2 / 2.0, clength, 0.0)
        self.length = float(clength)


class CompBallCutter(CompositeCutter):
    def __init__(self, diam2: float, clength: float):
        super().__init__()
        self.addCutter(BallCutter(diam2, clength), diam2 / 2.0, clength, 0.0)
        self.length = float(clength)


class CylConeCutter(CompositeCutter):
    """Flat centre of diameter diam1, cone of half-angle `angle` out to diam2."""

    def __init__(self, diam1: float, diam2: float, angle: float):
        super().__init__()
        cone_offset = -(diam1 / 2) / math.tan(angle)
        cyl_height = 0.0
        cone_height = (diam2 / 2.0) / math.tan(angle) + cone_offset
        self.addCutter(CylCutter(diam1, 1), diam1 / 2.0, cyl_height, 0.0)
        self.addCutter(ConeCutter(diam2, angle), diam2 / 2.0, cone_height, cone_offset)
        self.addCutter(CylCutter(diam2, 20), diam2 / 2.0, (diam2 / 2.0) / math.tan(angle) + 20, cone_height)
        self.length = cyl_height + cone_height + 10


class BallConeCutter(CompositeCutter):
    """Ball of diameter diam1 inside a cone of half-angle `angle` out to diam2,
    tangent where they meet."""

    def __init__(self, diam1: float, diam2: float, angle: float):
        super().__init__()
        radius1 = diam1 / 2.0
        radius2 = diam2 / 2.0
        rcontact = radius1 * math.cos(angle)
        height1 = radius1 - math.sqrt(radius1 * radius1 - rcontact * rcontact)
        cone_offset = -((rcontact) / math.tan(angle) - height1)
        height2 = radius2 / math.tan(angle) + cone_offset
        shaft_offset = height2
        self.addCutter(BallCutter(diam1, 1), rcontact, height1, 0.0)
        self.addCutter(ConeCutter(diam2, angle), diam2 / 2.0, height2, cone_offset)
        self.addCutter(CylCutter(diam2, 20), diam2 / 2.0, height2 + 20, shaft_offset)
        self.length = 30.0


class BullConeCutter(CompositeCutter):
    """Bull of diameter diam1 / corner radius radius1 inside a cone out to diam2."""

    def __init__(self, diam1: float, radius1: float, diam2: float, angle: float):
        super().__init__()
        h1 = radius1 * math.sin(angle)
        rad = math.sqrt(radius1 * radius1 - h1 * h1)
        rcontact = (diam1 / 2.0) - radius1 + rad
        cone_offset = -(rcontact / math.tan(angle) - (radius1 - h1))
        height1 = radius1 - h1
        height2 = (diam2 / 2.0) / math.tan(angle) + cone_offset
        shaft_offset = height2
        self.addCutter(BullCutter(diam1, radius1, 1.0), rcontact, height1, 0.0)
        self.addCutter(ConeCutter(diam2, angle), diam2 / 2.0, height2, cone_offset)
        self.addCutter(CylCutter(diam2, 20), diam2 / 2.0, height2 + 20, shaft_offset)
        self.length = 30.0


class ConeConeCutter(CompositeCutter):
    """Cone (diam1, angle1) below a cone (diam2, angle2)."""

    def __init__(self, diam1: float, angle1: float, diam2: float, angle2: float):
        super().__init__()
        height1 = (diam1 / 2.0) / math.tan(angle1)
        tmp = (diam1 / 2.0) / math.tan(angle2)
        cone_offset = -(tmp - height1)
        height2 = (diam2 / 2.0) / math.tan(angle2) + cone_offset
        shaft_offset = height2
        self.addCutter(ConeCutter(diam1, angle1), diam1 / 2.0, height1, 0.0)
        self.addCutter(ConeCutter(diam2, angle2), diam2 / 2.0, height2, cone_offset)
        self.addCutter(CylCutter(diam2, 20), diam2 / 2.0, height2 + 20, shaft_offset)
        self.length = 30.0


def standard_cutters():
    """The five cutters of the 1M-triangle precision workload, by name."""
    return {
        "cyl": CylCutter(6.0, 20.0),
        "ball": BallCutter(6.0, 20.0),
        "bull": BullCutter(6.0, 1.0, 20.0),
        "cone": ConeCutter(6.0, math.pi / 4, 20.0),
        "ballcone": BallConeCutter(2.0, 6.0, math.pi / 4),
    }
