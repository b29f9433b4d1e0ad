"""Seeded synthetic meshes, CL rasters, fibers and paths.

No public dataset is involved in the drop-/push-cutter benchmarks, so these
generators define the workloads.  All randomness comes from splitmix64
(output k of stream `seed` is mix(seed + (k+1)*golden)), so every output is
a pure function of (seed, index) and identical on any host; uniforms are
(x >> 11) * 2**-53 and normals use Box-Muller.

Workloads (sizes as used by the tests and the benchmark):
  heightfield_c1   128x128-vertex bump field on [0,100]^2 -> 32,258 triangles
  mesh_c2          512x1024 jittered bump field + hemisphere r=30 + 2-triangle
                   plate -> exactly 1,048,576 triangles
  raster           CL points on a regular xy raster at a given start z
  sphere_torus     sphere-on-plate + torus (R=25, r=8) for the push-cutter
  batch_jobs       64 drop-cutter jobs of uneven mesh and point counts
                   (heightfield / sphere / box-with-fillet meshes, all five
                   cutter families, diameters 1-20 mm)
"""
from __future__ import annotations

import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, start: int = 0) -> np.ndarray:
    """Outputs start..start+n-1 of the splitmix64 stream with this seed."""
    with np.errstate(over="ignore"):
        k = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int, start: int = 0) -> np.ndarray:
    """U[0,1) doubles from the top 53 bits."""
    return (splitmix64(seed, n, start) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def normal(seed: int, n: int, start: int = 0) -> np.ndarray:
    """N(0,1) by Box-Muller from consecutive uniform pairs."""
    u = uniform(seed, 2 * n, 2 * start)
    u1 = 1.0 - u[0::2]
    u2 = u[1::2]
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


def bumps(seed: int, count: int = 8):
    """Gaussian bump parameters, drawn per bump in the order (A, sigma, cx, cy):
    A ~ U[2,15] mm, sigma ~ U[5,20] mm, centre ~ U[0,100]^2."""
    u = uniform(seed, 4 * count).reshape(count, 4)
    A = 2.0 + 13.0 * u[:, 0]
    s = 5.0 + 15.0 * u[:, 1]
    cx = 100.0 * u[:, 2]
    cy = 100.0 * u[:, 3]
    return A, s, cx, cy


def bump_height(x, y, params, base: float = 10.0):
    A, s, cx, cy = params
    z = np.full(np.broadcast(x, y).shape, base, dtype=np.float64)
    for k in range(len(A)):
        z = z + A[k] * np.exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / (2.0 * s[k] ** 2))
    return z


def grid_triangles(X: np.ndarray, Y: np.ndarray, Z: np.ndarray) -> np.ndarray:
    """Triangulate a vertex grid (arrays indexed [j, i], i along x).  Cell
    (i, j) gives (p00, p10, p11) and (p00, p11, p01); cells in row-major order
    (j outer, i inner)."""
    P = np.stack([X, Y, Z], axis=-1)
    p00 = P[:-1, :-1]
    p10 = P[:-1, 1:]
    p11 = P[1:, 1:]
    p01 = P[1:, :-1]
    t1 = np.concatenate([p00, p10, p11], axis=-1)
    t2 = np.concatenate([p00, p11, p01], axis=-1)
    return np.stack([t1, t2], axis=2).reshape(-1, 9)


def heightfield(nx: int, ny: int, seed: int = 1, jitter: float = 0.0, jitter_seed: int = 2,
                size: float = 100.0, nbumps: int = 8) -> np.ndarray:
    """Bump heightfield with nx x ny vertices over [0,size]^2."""
    xs = np.linspace(0.0, size, nx)
    ys = np.linspace(0.0, size, ny)
    X, Y = np.meshgrid(xs, ys)
    Z = bump_height(X, Y, bumps(seed, nbumps))
    if jitter > 0.0:
        n = nx * ny
        g = normal(jitter_seed, 3 * n).reshape(3, ny, nx) * jitter
        X = X + g[0]
        Y = Y + g[1]
        Z = Z + g[2]
    return grid_triangles(X, Y, Z)


def heightfield_c1() -> np.ndarray:
    """128x128 vertices on [0,100]^2 (h = 100/127): 32,258 triangles."""
    return heightfield(128, 128, seed=1)


def hemisphere(cx: float, cy: float, cz: float, r: float, naz: int = 52, nrings: int = 30) -> np.ndarray:
    """Upper hemisphere: a pole fan of naz triangles, then nrings-1 bands of
    2*naz triangles; ring k at polar angle k*(pi/2)/nrings."""
    tris = []
    th = np.arange(nrings + 1) * (math.pi / 2.0) / nrings
    ph = 2.0 * math.pi * np.arange(naz) / naz

    def v(k, m):
        m = m % naz
        return (cx + r * math.sin(th[k]) * math.cos(ph[m]), cy + r * math.sin(th[k]) * math.sin(ph[m]),
                cz + r * math.cos(th[k]))

    pole = (cx, cy, cz + r)
    for m in range(naz):
        tris.append(pole + v(1, m) + v(1, m + 1))
    for k in range(1, nrings):
        for m in range(naz):
            a, b, c, d = v(k, m), v(k, m + 1), v(k + 1, m + 1), v(k + 1, m)
            tris.append(a + d + c)
            tris.append(a + c + b)
    return np.array(tris, dtype=np.float64)


def plate(z: float, x0: float = 0.0, x1: float = 100.0, y0: float = 0.0, y1: float = 100.0) -> np.ndarray:
    return np.array([[x0, y0, z, x1, y0, z, x1, y1, z], [x0, y0, z, x1, y1, z, x0, y1, z]], dtype=np.float64)


def mesh_c2() -> np.ndarray:
    """Exactly 1,048,576 triangles: 512x1024-vertex bump field with vertex
    jitter N(0, 0.01 mm) on x, y and z (1,045,506 triangles), a hemisphere
    r=30 centred (50,50,10) with 52 azimuth x 30 rings (3,068 triangles) and
    a 2-triangle plate at z=10 over [0,100]^2."""
    hf = heightfield(512, 1024, seed=1, jitter=0.01, jitter_seed=2)
    hs = hemisphere(50.0, 50.0, 10.0, 30.0)
    t = np.concatenate([hf, hs, plate(10.0)], axis=0)
    assert t.shape[0] == 1 << 20
    return t


def raster(nx: int, ny: int, step: float, z0: float = -50.0, x0: float = 0.0, y0: float = 0.0) -> np.ndarray:
    """CL points x = x0 + step*i, y = y0 + step*j (j outer, i inner)."""
    xs = x0 + step * np.arange(nx)
    ys = y0 + step * np.arange(ny)
    X, Y = np.meshgrid(xs, ys)
    return np.stack([X.ravel(), Y.ravel(), np.full(X.size, z0)], axis=1)


def raster_c1() -> np.ndarray:
    return raster(200, 200, 0.5)


def raster_c2() -> np.ndarray:
    return raster(1000, 1000, 0.1)


def subsample(n_total: int, n: int, seed: int) -> np.ndarray:
    """Seeded sample of n distinct indices out of n_total, sorted."""
    key = splitmix64(seed, n_total)
    return np.sort(np.argsort(key, kind="stable")[:n])


def torus(cx, cy, cz, R, r, nu, nv) -> np.ndarray:
    """Torus around the z axis, nu x nv quads -> 2*nu*nv triangles."""
    u = 2.0 * math.pi * np.arange(nu) / nu
    w = 2.0 * math.pi * np.arange(nv) / nv
    U, W = np.meshgrid(u, w, indexing="ij")
    X = cx + (R + r * np.cos(W)) * np.cos(U)
    Y = cy + (R + r * np.cos(W)) * np.sin(U)
    Z = cz + r * np.sin(W)
    P = np.stack([X, Y, Z], axis=-1)
    Pn = np.roll(P, -1, axis=0)
    Pm = np.roll(P, -1, axis=1)
    Pnm = np.roll(Pn, -1, axis=1)
    t1 = np.concatenate([P, Pn, Pnm], axis=-1)
    t2 = np.concatenate([P, Pnm, Pm], axis=-1)
    return np.stack([t1, t2], axis=2).reshape(-1, 9)


def sphere(cx, cy, cz, r, naz, nrings) -> np.ndarray:
    """Full UV sphere: a north pole fan, nrings-2 bands of two triangles per
    quad, a south pole fan (vertex (k, m) at polar angle k pi / nrings and
    azimuth 2 pi m / naz)."""
    th = np.arange(nrings + 1) * math.pi / nrings
    ph = 2.0 * math.pi * np.arange(naz) / naz
    ct, st = np.cos(th), np.sin(th)
    cp, sp = np.cos(ph), np.sin(ph)
    V = np.stack([cx + r * st[:, None] * cp[None, :], cy + r * st[:, None] * sp[None, :],
                  np.broadcast_to(cz + r * ct[:, None], (nrings + 1, naz))], axis=-1)  # [k, m, xyz]
    Vn = np.roll(V, -1, axis=1)  # vertex (k, m + 1)
    north = np.broadcast_to(np.array([cx, cy, cz + r]), (naz, 3))
    south = np.broadcast_to(np.array([cx, cy, cz - r]), (naz, 3))
    fan_n = np.concatenate([north, V[1], Vn[1]], axis=1)
    a, b = V[1:nrings - 1], Vn[1:nrings - 1]
    c, d = Vn[2:nrings], V[2:nrings]
    band = np.stack([np.concatenate([a, d, c], axis=-1), np.concatenate([a, c, b], axis=-1)], axis=2)
    fan_s = np.concatenate([south, Vn[nrings - 1], V[nrings - 1]], axis=1)
    return np.concatenate([fan_n, band.reshape(-1, 9), fan_s], axis=0)


def sphere_torus(scale: int = 1) -> np.ndarray:
    """Sphere-on-plate (sphere r=20 at (50,50,20), plate z=0 over [0,100]^2)
    plus a torus R=25, r=8 around the sphere at z=8.  scale=1 gives ~500k
    triangles; smaller scales give test-sized meshes."""
    if scale == 1:
        s = sphere(50.0, 50.0, 20.0, 20.0, 400, 300)
        t = torus(50.0, 50.0, 8.0, 25.0, 8.0, 520, 250)
    else:
        s = sphere(50.0, 50.0, 20.0, 20.0, 24 * scale, 16 * scale)
        t = torus(50.0, 50.0, 8.0, 25.0, 8.0, 32 * scale, 12 * scale)
    return np.concatenate([s, t, plate(0.0)], axis=0)


def fibers(direction: int, z: float, lo: float, hi: float, n: int, ext_lo: float, ext_hi: float) -> np.ndarray:
    """n fibers at height z, evenly spaced over [lo, hi] across, spanning
    [ext_lo, ext_hi] along (direction 0 = X-fibers, 1 = Y-fibers)."""
    c = np.linspace(lo, hi, n)
    f = np.zeros((n, 6))
    if direction == 0:
        f[:, 0] = ext_lo
        f[:, 3] = ext_hi
        f[:, 1] = c
        f[:, 4] = c
    else:
        f[:, 1] = ext_lo
        f[:, 4] = ext_hi
        f[:, 0] = c
        f[:, 3] = c
    f[:, 2] = z
    f[:, 5] = z
    return f


def box_fillet(nx: int, ny: int, size: float = 100.0, h: float = 20.0, r: float = 5.0) -> np.ndarray:
    """A box with rounded top edges standing on a plate, as an nx x ny
    heightfield over [0,size]^2: flat top of height h over the middle of the
    square (60% x 40% of it), quarter-circle fillets of radius r along its top
    edges, then a vertical drop to the plate at z = 0 (one grid cell wide)."""
    xs = np.linspace(0.0, size, nx)
    ys = np.linspace(0.0, size, ny)
    X, Y = np.meshgrid(xs, ys)
    x0, x1 = 0.2 * size + r, 0.8 * size - r
    y0, y1 = 0.3 * size + r, 0.7 * size - r
    dx = np.maximum(np.maximum(x0 - X, X - x1), 0.0)
    dy = np.maximum(np.maximum(y0 - Y, Y - y1), 0.0)
    q = np.sqrt(dx * dx + dy * dy)
    Z = np.where(q <= 0.0, h, np.where(q < r, h - r + np.sqrt(np.maximum(r * r - q * q, 0.0)), 0.0))
    return grid_triangles(X, Y, Z)


def mesh_of_size(kind: str, n: int, seed: int) -> np.ndarray:
    """About n triangles from one of the batch generators: 'heightfield' (a
    bump field), 'sphere' (a UV sphere r=40 on nothing), 'box' (box_fillet)."""
    if kind == "sphere":
        # 2 naz (nrings - 1) triangles with naz = 2 nrings
        nr = max(3, int(round(math.sqrt(n / 4.0))))
        return sphere(50.0, 50.0, 0.0, 40.0, 2 * nr, nr)
    side = max(3, int(round(math.sqrt(n / 2.0))) + 1)
    if kind == "box":
        return box_fillet(side, side)
    return heightfield(side, side, seed=seed)


def batch_jobs(seed: int = 3, njobs: int = 64, n_range=(1e3, 2e6), m_range=(1e3, 4e6), d_range=(1.0, 20.0)):
    """Seeded job specs of the batching workload: per job a mesh generator
    (uniform over heightfield, sphere, box), a triangle count N ~
    log-uniform(n_range), a CL point count M ~ log-uniform(m_range) on a
    raster over the mesh's bbox, a cutter family uniform over the five
    (cyl, ball, bull, cone, ball-cone) and a diameter d ~ U(d_range) (bull
    corner d/6, cones 45 deg, ball-cone d/3 inside d).  Returns a list of
    dicts; build_batch_job() makes the mesh and points."""
    u = uniform(seed, 6 * njobs).reshape(njobs, 6)
    kinds = ("heightfield", "sphere", "box")
    cutters_ = ("cyl", "ball", "bull", "cone", "ballcone")
    out = []
    for k in range(njobs):
        N = int(round(math.exp(math.log(n_range[0]) + u[k, 0] * (math.log(n_range[1]) - math.log(n_range[0])))))
        M = int(round(math.exp(math.log(m_range[0]) + u[k, 1] * (math.log(m_range[1]) - math.log(m_range[0])))))
        out.append({"job": k, "mesh": kinds[min(int(u[k, 2] * 3), 2)], "N": N, "M": M,
                    "cutter": cutters_[min(int(u[k, 3] * 5), 4)],
                    "d": d_range[0] + (d_range[1] - d_range[0]) * u[k, 4], "seed": seed * 1000 + k})
    return out


def batch_cutter(name: str, d: float):
    from . import cutters as cu
    L = max(20.0, 2.0 * d)
    return {"cyl": lambda: cu.CylCutter(d, L), "ball": lambda: cu.BallCutter(d, L),
            "bull": lambda: cu.BullCutter(d, d / 6.0, L), "cone": lambda: cu.ConeCutter(d, math.pi / 4, L),
            "ballcone": lambda: cu.BallConeCutter(d / 3.0, d, math.pi / 4)}[name]()


def batch_points(tris: np.ndarray, M: int, margin: float) -> np.ndarray:
    """About M points on a raster over the mesh bbox widened by margin,
    starting 10 mm below the mesh."""
    p = tris.reshape(-1, 3)
    lo, hi = p.min(axis=0), p.max(axis=0)
    w, h = hi[0] - lo[0] + 2 * margin, hi[1] - lo[1] + 2 * margin
    nx = max(1, int(round(math.sqrt(M * w / h))))
    ny = max(1, int(round(M / nx)))
    xs = lo[0] - margin + (np.arange(nx) + 0.5) * (w / nx)
    ys = lo[1] - margin + (np.arange(ny) + 0.5) * (h / ny)
    X, Y = np.meshgrid(xs, ys)
    return np.stack([X.ravel(), Y.ravel(), np.full(X.size, lo[2] - 10.0)], axis=1)


def serving_requests(seed: int = 5, n: int = 200, rate: float = 200.0, nmeshes: int = 8):
    """Seeded request stream of the serving workload: Poisson arrivals at
    `rate` per second; BatchDropCutter and AdaptivePathDropCutter requests
    1:1; a mesh uniform over `nmeshes`; a cutter family uniform over the five
    with diameter U[2, 12] mm; drops with log-uniform 100 .. 1,000,000 raster
    points over the mesh bbox; adaptive paths of total length U[10, 500] mm
    (a zig-zag of line spans across the mesh), sampling U[0.1, 1] mm,
    minimum sampling 0.01 mm.  Returns dicts; points and spans are made by
    serving_payload() against the mesh's bbox."""
    u = uniform(seed, 8 * n).reshape(n, 8)
    t = np.cumsum(-np.log(1.0 - u[:, 0]) / rate)
    cutters_ = ("cyl", "ball", "bull", "cone", "ballcone")
    out = []
    for k in range(n):
        r = {"t": float(t[k]), "kind": "drop" if u[k, 1] < 0.5 else "adaptive", "mesh": int(u[k, 2] * nmeshes),
             "cutter": cutters_[min(int(u[k, 3] * 5), 4)], "d": 2.0 + 10.0 * u[k, 4], "u": u[k, 5:].copy()}
        if r["kind"] == "drop":
            r["M"] = int(round(math.exp(math.log(100) + u[k, 5] * (math.log(1e6) - math.log(100)))))
        else:
            r["length"] = 10.0 + 490.0 * u[k, 5]
            r["sampling"] = 0.1 + 0.9 * u[k, 6]
            r["min_sampling"] = 0.01
        out.append(r)
    return out


def serving_meshes(seed: int = 5, n: int = 8):
    """The resident meshes of the serving workload: generator cycling over
    heightfield / sphere / box, N ~ log-uniform 10,000 .. 2,000,000."""
    u = uniform(seed + 1, n)
    kinds = ("heightfield", "sphere", "box")
    return [mesh_of_size(kinds[k % 3], int(round(math.exp(math.log(1e4) + u[k] * (math.log(2e6) - math.log(1e4))))),
                         seed * 100 + k) for k in range(n)]


def serving_payload(req, tris):
    """CL points (drop) or spans (adaptive path) of a request over a mesh."""
    p = tris.reshape(-1, 3)
    lo, hi = p.min(axis=0), p.max(axis=0)
    z0 = lo[2] - 10.0
    if req["kind"] == "drop":
        pts = batch_points(tris, req["M"], 0.0)
        pts[:, 2] = z0
        return pts
    w, h = hi[0] - lo[0], hi[1] - lo[1]
    L = req["length"]
    nlines = max(1, int(math.ceil(L / max(w, 1e-3))))
    spans = []
    left = L
    for j in range(nlines):
        seg = min(w, left)
        left -= seg
        y = lo[1] + h * (j + 0.5) / nlines
        a, b = (lo[0], lo[0] + seg) if j % 2 == 0 else (hi[0], hi[0] - seg)
        spans.append([0, a, y, z0, b, y, z0, 0, 0, 0, 0])
    return np.array(spans, dtype=np.float64)
