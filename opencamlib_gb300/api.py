"""Operation classes with the reference's Python API (src/pythonlib):
geometry (Point, CLPoint, CCPoint, Triangle, STLSurf, Bbox, Line, Arc, Path),
Fiber/Interval, and BatchDropCutter, PathDropCutter, AdaptivePathDropCutter,
BatchPushCutter.  run() calls the CUDA library through DeviceMesh; the
triangles of an STLSurf are uploaded once per surface and cached.
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi
from ._native import DeviceMesh, line_filter, stl_read

__all__ = ["Point", "CCPoint", "CLPoint", "Triangle", "STLSurf", "STLReader", "Bbox", "Line", "Arc", "Path",
           "Interval", "Fiber", "BatchDropCutter", "PathDropCutter", "AdaptivePathDropCutter", "BatchPushCutter",
           "LineCLFilter", "CCType", "Waterline", "AdaptiveWaterline"]


class CCType:
    """ocl::CCType values (src/geo/ccpoint.hpp:33-39)."""


for _i, _n in enumerate(_abi.CCTYPE_NAMES):
    setattr(CCType, _n, _i)


class Point:
    __slots__ = ("x", "y", "z")

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def __add__(self, o):
        return Point(self.x + o.x, self.y + o.y, self.z + o.z)

    def __sub__(self, o):
        return Point(self.x - o.x, self.y - o.y, self.z - o.z)

    def __mul__(self, a):
        return Point(self.x * a, self.y * a, self.z * a)

    __rmul__ = __mul__

    def dot(self, o):
        return self.x * o.x + self.y * o.y + self.z * o.z

    def cross(self, p):
        return Point(self.y * p.z - self.z * p.y, self.z * p.x - self.x * p.z, self.x * p.y - self.y * p.x)

    def norm(self):
        return math.sqrt(self.x * self.x + self.y * self.y + self.z * self.z)

    def xyNorm(self):
        return math.sqrt(self.x * self.x + self.y * self.y)

    def normalize(self):
        n = self.norm()
        if n != 0.0:
            self.x, self.y, self.z = self.x * (1 / n), self.y * (1 / n), self.z * (1 / n)

    def str(self):
        return f"({self.x}, {self.y}, {self.z})"

    __repr__ = str

    def __eq__(self, o):
        return isinstance(o, Point) and self.x == o.x and self.y == o.y and self.z == o.z

    # rotations about the x, y, z axes (src/geo/point.cpp:105-134)
    def xRotate(self, theta):
        self.x, self.y, self.z = _rotate3(_rx(theta), self.x, self.y, self.z)

    def yRotate(self, theta):
        self.x, self.y, self.z = _rotate3(_ry(theta), self.x, self.y, self.z)

    def zRotate(self, theta):
        self.x, self.y, self.z = _rotate3(_rz(theta), self.x, self.y, self.z)


def _rx(t):
    c, s = math.cos(t), math.sin(t)
    return (1.0, 0.0, 0.0, 0.0, c, -s, 0.0, s, c)


def _ry(t):
    c, s = math.cos(t), math.sin(t)
    return (c, 0.0, s, 0.0, 1.0, 0.0, -s, 0.0, c)


def _rz(t):
    c, s = math.cos(t), math.sin(t)
    return (c, -s, 0.0, s, c, 0.0, 0.0, 0.0, 1.0)


def _rotate3(m, x, y, z):
    """Point::matrixRotate: each row of the matrix times (x, y, z), summed
    left to right (scalars or numpy arrays; no fused multiply-add)."""
    a, b, c, d, e, f, g, h, i = m
    return a * x + b * y + c * z, d * x + e * y + f * z, g * x + h * y + i * z


class CCPoint(Point):
    __slots__ = ("type",)

    def __init__(self, x=0.0, y=0.0, z=0.0, t=0):
        super().__init__(x, y, z)
        self.type = int(t)

    def str(self):
        return f"CC({self.x}, {self.y}, {self.z}, t={self.type})"

    __repr__ = str


class CLPoint(Point):
    __slots__ = ("_cc",)

    def __init__(self, x=0.0, y=0.0, z=0.0, cc=None):
        super().__init__(x, y, z)
        self._cc = cc if cc is not None else CCPoint()

    def cc(self):
        return self._cc

    def getCC(self):
        return self._cc

    def str(self):
        return f"CL({self.x}, {self.y}, {self.z}) cc={self._cc.str()}"

    __repr__ = str


class Bbox:
    def __init__(self, minx=0, maxx=0, miny=0, maxy=0, minz=0, maxz=0):
        self.minpt = Point(minx, miny, minz)
        self.maxpt = Point(maxx, maxy, maxz)

    def __getitem__(self, i):
        return [self.minpt.x, self.maxpt.x, self.minpt.y, self.maxpt.y, self.minpt.z, self.maxpt.z][i]


class Triangle:
    def __init__(self, p1=None, p2=None, p3=None):
        if p1 is None:
            p1, p2, p3 = Point(1, 0, 0), Point(0, 1, 0), Point(0, 0, 1)
        self.p = [Point(p1.x, p1.y, p1.z), Point(p2.x, p2.y, p2.z), Point(p3.x, p3.y, p3.z)]

    def getPoints(self):
        return list(self.p)

    def rotate(self, xr, yr, zr):
        """Triangle::rotate (src/geo/triangle.cpp:130-138)."""
        for q in self.p:
            q.xRotate(xr)
            q.yRotate(yr)
            q.zRotate(zr)

    def array(self):
        return [c for q in self.p for c in (q.x, q.y, q.z)]


class STLSurf:
    """Triangle list (src/geo/stlsurf.hpp:38-56).  addTriangle appends; the
    device copy is made on first use and reused until the surface changes."""

    def __init__(self, tris=None):
        self._rows = []
        self._arr = None if tris is None else np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 9)
        self._dev = {}

    def addTriangle(self, t: Triangle):
        self._materialize_rows()
        self._rows.append(t.array())
        self._arr = None
        self._dev = {}

    def _extend(self, tris):
        # many addTriangle calls at once: tris is (n, 9)
        tris = np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 9)
        if len(tris) == 0:
            return
        self._arr = tris.copy() if self.size() == 0 else np.concatenate([self.array(), tris])
        self._rows = []
        self._dev = {}

    def _materialize_rows(self):
        if self._arr is not None and not self._rows:
            self._rows = self._arr.tolist()
            self._arr = None

    def array(self):
        if self._arr is None:
            self._arr = np.array(self._rows, dtype=np.float64).reshape(-1, 9)
        return self._arr

    def size(self):
        return int(self.array().shape[0])

    def rotate(self, xr, yr, zr):
        """STLSurf::rotate (src/geo/stlsurf.cpp:44-55): every vertex rotated
        about x, then y, then z; the device copy is made again on next use."""
        a = self.array().reshape(-1, 3).copy()
        x, y, z = a[:, 0], a[:, 1], a[:, 2]
        for m in (_rx(xr), _ry(yr), _rz(zr)):
            x, y, z = _rotate3(m, x, y, z)
        self._arr = np.stack([x, y, z], axis=1).reshape(-1, 9)
        self._rows = []
        self._dev = {}

    def getTriangles(self):
        a = self.array()
        return [Triangle(Point(*r[0:3]), Point(*r[3:6]), Point(*r[6:9])) for r in a]

    def getBounds(self):
        a = self.array().reshape(-1, 3)
        if a.size == 0:
            return [0.0] * 6
        mn, mx = a.min(axis=0), a.max(axis=0)
        return [mn[0], mx[0], mn[1], mx[1], mn[2], mx[2]]

    @property
    def bb(self):
        return Bbox(*self.getBounds())

    def device(self, bucket_size=1) -> DeviceMesh:
        m = self._dev.get(bucket_size)
        if m is None:
            m = DeviceMesh(self.array(), bucket_size)
            self._dev[bucket_size] = m
        return m

    def str(self):
        return f"STLSurf(N={self.size()})"

    __repr__ = str


class STLReader:
    """STLReader(filename, surface) adds the file's triangles to the surface
    (src/geo/stlreader.cpp:35-37, 57-150; the file is parsed by the library's
    host code).  A file that cannot be read adds nothing, as in the reference."""

    def __init__(self, filename=None, surface=None):
        if filename is not None and surface is not None:
            surface._extend(stl_read(filename, strict=False))


class LineCLFilter:
    """LineCLFilter (src/common/lineclfilter.cpp, Python API of
    src/pythonlib/ocl_algo.cpp:172-179): addCLPoint copies, run() keeps the
    points the filter selects (selection in the library), getCLPoints()
    returns them."""

    def __init__(self):
        self._pts = []
        self._tol = 0.0

    def addCLPoint(self, p):
        cc = p.getCC() if isinstance(p, CLPoint) else None
        self._pts.append(CLPoint(p.x, p.y, p.z, cc))

    def setTolerance(self, tol):
        self._tol = float(tol)

    def run(self):
        if len(self._pts) < 2:
            return
        xyz = np.array([[p.x, p.y, p.z] for p in self._pts], dtype=np.float64)
        self._pts = [self._pts[i] for i in line_filter(xyz, self._tol)]

    def getCLPoints(self):
        return list(self._pts)


class Line:
    def __init__(self, p1: Point, p2: Point):
        self.p1, self.p2 = p1, p2

    def row(self):
        return [0, self.p1.x, self.p1.y, self.p1.z, self.p2.x, self.p2.y, self.p2.z, 0, 0, 0, 0]


class Arc:
    def __init__(self, p1: Point, p2: Point, c: Point, dir: bool):
        self.p1, self.p2, self.c, self.dir = p1, p2, c, bool(dir)

    def row(self):
        return [1, self.p1.x, self.p1.y, self.p1.z, self.p2.x, self.p2.y, self.p2.z, self.c.x, self.c.y, self.c.z,
                1.0 if self.dir else 0.0]


class Path:
    def __init__(self):
        self.span_list = []

    def append(self, s):
        self.span_list.append(s)

    def getSpans(self):
        return list(self.span_list)

    def array(self):
        return np.array([s.row() for s in self.span_list], dtype=np.float64).reshape(-1, _abi.SPAN_DOUBLES)


class Interval:
    def __init__(self, lower=0.0, upper=0.0):
        self.lower, self.upper = float(lower), float(upper)
        self.lower_cc = CCPoint()
        self.upper_cc = CCPoint()

    def empty(self):
        return self.lower == 0.0 and self.upper == 0.0

    def str(self):
        return f"I [{self.lower} , {self.upper} ]"

    __repr__ = str


class Fiber:
    def __init__(self, p1: Point, p2: Point):
        self.p1, self.p2 = Point(p1.x, p1.y, p1.z), Point(p2.x, p2.y, p2.z)
        d = self.p2 - self.p1
        d.normalize()
        self.dir = d
        self.ints = []

    def point(self, t):
        return self.p1 + (self.p2 - self.p1) * t

    def getInts(self):
        return list(self.ints)

    def upperCLPoint(self, n):
        return self.point(self.ints[n].upper)

    def lowerCLPoint(self, n):
        return self.point(self.ints[n].lower)

    def printInts(self):
        for n, i in enumerate(self.ints):
            print(f"{n}: [ {i.lower} , {i.upper} ]")

    def row(self):
        return [self.p1.x, self.p1.y, self.p1.z, self.p2.x, self.p2.y, self.p2.z]


class _Operation:
    """Common setters of the reference's Operation (src/algo/operation.hpp:43-138)."""

    def __init__(self):
        self.surf = None
        self.cutter = None
        self.nthreads = 0
        self.bucketSize = 1
        self.sampling = 0.1
        self.nCalls = 0
        self.precision = "mixed"
        self.stats = None

    def setSTL(self, s: STLSurf):
        self.surf = s

    def setCutter(self, c):
        self.cutter = c

    def setThreads(self, n):
        self.nthreads = int(n)  # accepted for API compatibility; the GPU ignores it

    def getThreads(self):
        return self.nthreads

    def setBucketSize(self, s):
        self.bucketSize = int(s)

    def getBucketSize(self):
        return self.bucketSize

    def getCalls(self):
        return self.nCalls

    def setSampling(self, s):
        self.sampling = float(s)

    def getSampling(self):
        return self.sampling

    def _mesh(self):
        if self.surf is None or self.cutter is None:
            raise RuntimeError("setSTL() and setCutter() must be called before run()")
        return self.surf.device(self.bucketSize)


def _clpoints(xyz, cc, ty):
    return [CLPoint(p[0], p[1], p[2], CCPoint(c[0], c[1], c[2], t)) for p, c, t in zip(xyz, cc, ty)]


class BatchDropCutter(_Operation):
    """BatchDropCutter (src/dropcutter/batchdropcutter.hpp:48-79)."""

    def __init__(self):
        super().__init__()
        self._pts = []

    def appendPoint(self, p):
        self._pts.append((p.x, p.y, p.z))

    def clearCLPoints(self):
        self._pts = []
        self._res = None

    def run(self):
        m = self._mesh()
        cl = np.array(self._pts, dtype=np.float64).reshape(-1, 3)
        z, cc, ty, st = m.drop(self.cutter, cl, self.precision)
        xyz = cl.copy()
        xyz[:, 2] = z
        self._res = (xyz, cc, ty)
        self.stats = st
        self.nCalls = int(st.pairs if st.pairs else st.refined)

    def getCLPoints(self):
        if getattr(self, "_res", None) is None:
            return [CLPoint(*p) for p in self._pts]
        return _clpoints(*self._res)


class PathDropCutter(_Operation):
    """PathDropCutter (src/dropcutter/pathdropcutter.hpp)."""

    def __init__(self):
        super().__init__()
        self.path = None
        self.minimumZ = 0.0
        self._res = None

    def setPath(self, p: Path):
        self.path = p

    def setZ(self, z):
        self.minimumZ = float(z)

    def getZ(self):
        return self.minimumZ

    def run(self):
        xyz, cc, ty, st = self._mesh().path_drop(self.cutter, self.path.array(), self.sampling, self.minimumZ)
        self._res = (xyz, cc, ty)
        self.stats = st

    def getCLPoints(self):
        return _clpoints(*self._res) if self._res else []

    getPoints = getCLPoints


class AdaptivePathDropCutter(PathDropCutter):
    """AdaptivePathDropCutter (src/dropcutter/adaptivepathdropcutter.hpp).
    Like the reference, the start z of the samples comes from the path; setZ
    is stored but not applied."""

    def __init__(self):
        super().__init__()
        self.min_sampling = 0.01
        self.cosLimit = 0.999

    def setMinSampling(self, s):
        if not s > 0.0:
            raise ValueError("min sampling must be > 0")
        self.min_sampling = float(s)

    def setCosLimit(self, c):
        self.cosLimit = float(c)

    def run(self):
        xyz, cc, ty, st = self._mesh().adaptive_path_drop(self.cutter, self.path.array(), self.sampling,
                                                          self.min_sampling, self.cosLimit)
        self._res = (xyz, cc, ty)
        self.stats = st


class BatchPushCutter(_Operation):
    """BatchPushCutter (src/algo/batchpushcutter.hpp); setXDirection() or
    setYDirection() selects the fiber direction."""

    def __init__(self):
        super().__init__()
        self.fibers = []
        self.x_direction = False
        self.y_direction = False

    def setXDirection(self):
        self.x_direction, self.y_direction = True, False

    def setYDirection(self):
        self.x_direction, self.y_direction = False, True

    def appendFiber(self, f: Fiber):
        g = Fiber(f.p1, f.p2)
        self.fibers.append(g)

    def reset(self):
        self.fibers = []

    def run(self):
        if not (self.x_direction or self.y_direction):
            raise RuntimeError("setXDirection() or setYDirection() must be called before run()")
        d = _abi.XFIBER if self.x_direction else _abi.YFIBER
        fib = np.array([f.row() for f in self.fibers], dtype=np.float64).reshape(-1, 6)
        res, st = self._mesh().push(self.cutter, d, fib)
        self.stats = st
        self.nCalls = int(st.pairs)
        for f, recs in zip(self.fibers, res):
            f.ints = []
            for lo, up, lcc, ucc, lt, ut in recs:
                i = Interval(lo, up)
                i.lower_cc = CCPoint(lcc[0], lcc[1], lcc[2], lt)
                i.upper_cc = CCPoint(ucc[0], ucc[1], ucc[2], ut)
                f.ints.append(i)

    def getFibers(self):
        return self.fibers

    def getCLPoints(self):
        out = []
        for f in self.fibers:
            for n in range(len(f.ints)):
                out.append(f.lowerCLPoint(n))
                out.append(f.upperCLPoint(n))
        return out


class Waterline(_Operation):
    """Waterline (src/algo/waterline.hpp:41-88, Python binding
    src/pythonlib/ocl_algo.cpp:105-119): X and Y fibers at height z pushed on
    the GPU, woven on the host.  getLoops() gives a list of loops, each a
    list of Points; run2() gives the same loops as run()."""

    def __init__(self):
        super().__init__()
        self.zh = 0.0
        self.loops = []
        self.xfibers = []
        self.yfibers = []

    def setZ(self, z):
        self.zh = float(z)

    def _weave(self):
        return self._mesh().waterline(self.cutter, self.zh, self.sampling)

    def run(self):
        res, st = self._weave()
        self.stats = st
        self.nCalls = int(st.pairs)
        self.loops = [[Point(*p) for p in lp] for lp in res.loops]
        self.xfibers, self.yfibers = (self._fibers(res, d) for d in (0, 1))

    def run2(self):
        self.run()

    @staticmethod
    def _fibers(res, d):
        fib, off, iv, cc, ty = res.fibers(d)
        out = []
        for f in range(len(fib)):
            g = Fiber(Point(*fib[f, :3]), Point(*fib[f, 3:]))
            for k in range(int(off[f]), int(off[f + 1])):
                i = Interval(iv[k, 0], iv[k, 1])
                i.lower_cc = CCPoint(cc[k, 0, 0], cc[k, 0, 1], cc[k, 0, 2], int(ty[k, 0]))
                i.upper_cc = CCPoint(cc[k, 1, 0], cc[k, 1, 1], cc[k, 1, 2], int(ty[k, 1]))
                g.ints.append(i)
            out.append(g)
        return out

    def reset(self):
        self.loops, self.xfibers, self.yfibers = [], [], []

    def getLoops(self):
        return self.loops

    def getXFibers(self):
        return self.xfibers

    def getYFibers(self):
        return self.yfibers


class AdaptiveWaterline(Waterline):
    """AdaptiveWaterline (src/algo/adaptivewaterline.hpp:38-92): fibers
    bisected where the loops bend (setMinSampling, setCosLimit)."""

    def __init__(self):
        super().__init__()
        self.sampling = 1.0
        self.min_sampling = 0.1
        self.cosLimit = 0.999

    def setSampling(self, s):
        self.sampling = float(s)
        self.min_sampling = self.sampling / 10.0

    def setMinSampling(self, s):
        self.min_sampling = float(s)

    def setCosLimit(self, c):
        self.cosLimit = float(c)

    def _weave(self):
        return self._mesh().adaptive_waterline(self.cutter, self.zh, self.sampling, self.min_sampling, self.cosLimit)
