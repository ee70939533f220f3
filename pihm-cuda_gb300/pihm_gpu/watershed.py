"""Synthetic PIHM watersheds, deterministic from a seed.

The reference measures on no public dataset; its benchmark configurations
name a generator instead: a 10 x 10 km domain whose DEM is a 1 % tilted plane
plus 8 Gaussian hills (height U(20, 200) m, sigma U(0.5, 2) km), a triangular
mesh, a river network along the steepest-descent drainage to one outlet,
per-element soil drawn from the seed (Ksat lognormal 1e-6..1e-4 m/s,
porosity U(0.35, 0.5), van Genuchten alpha U(0.5, 5) /m and n U(1.2, 2.5),
depth U(2, 10) m, Manning n U(0.03, 0.1)), hourly precipitation that is wet
with probability 0.1 and then gamma(0.7, 3 mm/h), and a PET sinusoid peaking
at 0.3 mm/h.

Mesh.  Nodes sit on a jittered nx x ny grid (interior nodes moved up to 0.3
of a cell in x and y, boundary nodes only along their side).  Every cell is
split into two triangles along the diagonal that passes the Delaunay
empty-circumcircle test for the cell's four nodes, which gives exactly
2 (nx-1)(ny-1) elements (1,000 for 26 x 21 nodes) using only numpy arithmetic,
so the mesh is bit-identical on every machine.  Elements are emitted in a
seeded random order (mesh generators do not emit locality-sorted elements; the
GPU library renumbers them itself).

Derived geometry restates the reference's initialisation formulas:
InitTopo (src/init_topo.c:6-52: area, centroid, zmin/zmax, edge lengths),
InitRiver (src/init_river.c:6-124: river topography, shape, material, the
negative neighbour ids of river edges, RiverEqWid) and InitSurfL
(src/initialize.c:385-458: neighbour centroids and distances), including the
reference's `pow(d, 2)` / summation order so that values agree with the
reference reading the same nodes.

River network.  Node elevations are depression-filled by a priority flood
from the single outlet over interior nodes (Barnes, Lehman & Mulla 2014,
"Priority-Flood", with an epsilon rise), each interior node drains to its
steepest-descent neighbour on the filled surface, and the `nriver` interior
nodes with the largest flow accumulation, with their downstream edges, form
the channel network (a tree rooted at the outlet).  The outlet segment gets
ZERO_DPTH_GRAD (-3) when its bed slopes down into the outlet, else CRIT_DPTH
(-4) (src/include/pihm_const.h:140-143).
"""
from __future__ import annotations

import dataclasses
import hashlib
import heapq
import math

import numpy as np

DEPRSTG = 1e-4
RIVDPTHMIN = 0.05
RECTANGLE, TRIANGLE, QUADRATIC, CUBIC = 1, 2, 3, 4
ZERO_DPTH_GRAD, CRIT_DPTH = -3, -4

ELEM_INT_FIELDS = ("nabr", "bc_type")
ELEM_F64_FIELDS = ("area", "zmin", "zmax", "edge", "nabrdist", "nabr_x",
                   "nabr_y", "depth", "ksath", "ksatv", "kinfv", "dinf",
                   "alpha", "beta", "porosity", "dmac", "kmach", "kmacv",
                   "areafv", "areafh", "rough", "rzd")
RIVER_INT_FIELDS = ("down", "leftele", "rightele", "intrpl_ord",
                    "riverbc_type")
RIVER_F64_FIELDS = ("riv_area", "riv_zmin", "riv_zmax", "riv_zbed",
                    "riv_node_zmax", "riv_dist_left", "riv_dist_right",
                    "riv_depth", "riv_coeff", "riv_length", "riv_width",
                    "riv_rough", "riv_cwr", "riv_ksath", "riv_ksatv",
                    "riv_bedthick", "riv_porosity")
PER_EDGE = ("nabr", "bc_type", "edge", "nabrdist", "nabr_x", "nabr_y")
MESH_FIELDS = ELEM_INT_FIELDS + ELEM_F64_FIELDS + RIVER_INT_FIELDS + RIVER_F64_FIELDS


@dataclasses.dataclass
class Watershed:
    """One watershed in the reference's order: the arrays of pihm_gpu_mesh
    (include/pihm_gpu.h) plus the model controls the right-hand side reads."""
    nelem: int
    nriver: int
    arrays: dict
    surf_mode: int = 2
    riv_mode: int = 2
    stepsize: float = 60.0
    seed: int = 0
    x: np.ndarray | None = None   # element centroids (not read by the RHS)
    y: np.ndarray | None = None
    # the node mesh a generated watershed was built from (what an input deck
    # stores, pihm_gpu.deck.write_deck): node x, y, zmin, zmax, the element
    # node ids `tri` [nelem, 3] and the segment end nodes `from_n`, `to_n`,
    # all 0-based
    nodes: dict | None = None

    @property
    def neq(self) -> int:
        return 3 * self.nelem + 2 * self.nriver

    def digest(self) -> str:
        h = hashlib.sha256()
        for k in MESH_FIELDS:
            h.update(k.encode())
            h.update(np.ascontiguousarray(self.arrays[k]).tobytes())
        return h.hexdigest()

    def save(self, path: str) -> None:
        np.savez_compressed(path, nelem=self.nelem, nriver=self.nriver,
                            surf_mode=self.surf_mode, riv_mode=self.riv_mode,
                            stepsize=self.stepsize, seed=self.seed,
                            **{k: self.arrays[k] for k in MESH_FIELDS})

    @staticmethod
    def load(path: str) -> "Watershed":
        z = np.load(path)
        arrays = {k: np.ascontiguousarray(z[k]) for k in MESH_FIELDS}
        return Watershed(int(z["nelem"]), int(z["nriver"]), arrays,
                         int(z["surf_mode"]), int(z["riv_mode"]),
                         float(z["stepsize"]), int(z["seed"]))


# ----------------------------------------------------------------------------
# mesh
# ----------------------------------------------------------------------------

def _grid_shape(nelem: int) -> tuple[int, int]:
    """nx, ny with 2 (nx-1)(ny-1) == nelem (rounded to even), cells as square
    as a divisor pair allows."""
    cells = max(1, nelem // 2)
    best = (cells, 1)
    for b in range(1, int(math.isqrt(cells)) + 1):
        if cells % b == 0:
            best = (cells // b, b)
    a, b = best
    if a > 4 * b:  # prime-ish cell count: fall back to a near-square grid
        b = max(1, int(round(math.sqrt(cells))))
        a = max(1, cells // b)
    return a + 1, b + 1


def _dem(x, y, hills, length):
    """1 % plane falling towards +x plus Gaussian hills."""
    z = 100.0 + 0.01 * (length - x)
    for (cx, cy, h, s) in hills:
        z = z + h * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2.0 * s * s))
    return z


def _incircle(ax, ay, bx, by, cx, cy, dx, dy):
    """> 0 when d lies inside the circumcircle of the counter-clockwise a,b,c."""
    adx, ady = ax - dx, ay - dy
    bdx, bdy = bx - dx, by - dy
    cdx, cdy = cx - dx, cy - dy
    return ((adx * adx + ady * ady) * (bdx * cdy - cdx * bdy)
            - (bdx * bdx + bdy * bdy) * (adx * cdy - cdx * ady)
            + (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady))


def _triangulate(nx, ny, px, py):
    """Two counter-clockwise triangles per cell, Delaunay diagonal per cell."""
    i, j = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), indexing="xy")
    i = i.ravel()
    j = j.ravel()
    n00 = j * nx + i
    n10 = n00 + 1
    n01 = n00 + nx
    n11 = n01 + 1
    # diagonal n00-n11 is Delaunay when n01 is outside circle(n00, n10, n11)
    use_main = _incircle(px[n00], py[n00], px[n10], py[n10], px[n11], py[n11],
                         px[n01], py[n01]) <= 0.0
    t1 = np.where(use_main[:, None], np.stack([n00, n10, n11], 1),
                  np.stack([n00, n10, n01], 1))
    t2 = np.where(use_main[:, None], np.stack([n00, n11, n01], 1),
                  np.stack([n10, n11, n01], 1))
    return np.concatenate([t1, t2], 0).astype(np.int64)


def _scattered_points(nelem: int, length: float, rng):
    """Nodes of an unstructured mesh over the square: boundary nodes spaced
    along the four sides and interior nodes scattered one per stratum (a
    uniform point in each cell of a k x k stratification, some strata left
    empty), so that their Delaunay triangulation has about `nelem` triangles
    with the irregular node degrees and element sizes of a mesh generator's
    output rather than a grid's.  Returns px, py, interior, corner."""
    m = max(2, int(round(math.sqrt(nelem / 2.0))))           # boundary segments per side
    n_int = max(1, (nelem - 4 * m + 2) // 2)                 # triangles = 2 n_int + 4 m - 2
    k = int(math.ceil(math.sqrt(n_int)))
    cells = rng.permutation(k * k)[:n_int]
    ci, cj = cells % k, cells // k
    h = length / k
    ix = (ci + rng.uniform(0.05, 0.95, n_int)) * h
    iy = (cj + rng.uniform(0.05, 0.95, n_int)) * h
    t = np.arange(m) / m
    jit = rng.uniform(-0.3, 0.3, (4, m)) / m
    jit[:, 0] = 0.0                                          # corners stay put
    u = np.clip(t + jit, 0.0, 1.0)
    bx = np.concatenate([u[0] * length, np.full(m, length), (1.0 - u[2]) * length, np.zeros(m)])
    by = np.concatenate([np.zeros(m), u[1] * length, np.full(m, length), (1.0 - u[3]) * length])
    px = np.concatenate([bx, ix])
    py = np.concatenate([by, iy])
    interior = np.concatenate([np.zeros(4 * m, bool), np.ones(n_int, bool)])
    corner = np.zeros(px.shape[0], bool)
    corner[[0, m, 2 * m, 3 * m]] = True
    return px, py, interior, corner


def _delaunay(px, py):
    """Counter-clockwise Delaunay triangles of the nodes."""
    from scipy.spatial import Delaunay
    tri = Delaunay(np.stack([px, py], 1)).simplices.astype(np.int64)
    a = (px[tri[:, 1]] - px[tri[:, 0]]) * (py[tri[:, 2]] - py[tri[:, 0]]) - \
        (px[tri[:, 2]] - px[tri[:, 0]]) * (py[tri[:, 1]] - py[tri[:, 0]])
    tri[a < 0] = tri[a < 0][:, [0, 2, 1]]
    return tri


def _neighbours(tri):
    """nb[t, j] = triangle across the edge opposite node j, or -1."""
    nt = tri.shape[0]
    a = np.concatenate([tri[:, 1], tri[:, 2], tri[:, 0]])
    b = np.concatenate([tri[:, 2], tri[:, 0], tri[:, 1]])
    owner = np.tile(np.arange(nt), 3)
    slot = np.repeat(np.arange(3), nt)
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    key = lo * (tri.max() + 1) + hi
    order = np.argsort(key, kind="stable")
    ks = key[order]
    nb = -np.ones((nt, 3), np.int64)
    same = ks[1:] == ks[:-1]
    p = order[:-1][same]
    q = order[1:][same]
    nb[owner[p], slot[p]] = owner[q]
    nb[owner[q], slot[q]] = owner[p]
    return nb


# ----------------------------------------------------------------------------
# drainage
# ----------------------------------------------------------------------------

def _node_adjacency(tri, nnode):
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    e = np.concatenate([e, e[:, ::-1]])
    key = np.sort(e[:, 0] * nnode + e[:, 1])
    key = key[np.concatenate([[True], key[1:] != key[:-1]])]
    u = key // nnode
    v = key % nnode
    start = np.searchsorted(u, np.arange(nnode + 1))
    return u, v, start


def _drainage(z, px, py, interior, outlet, u, v, start):
    """Priority-flood (epsilon) from `outlet` over interior nodes, then
    steepest descent on the filled surface.  Returns down[node] (-1 for the
    outlet and for nodes outside the drainage graph) and the fill."""
    nnode = z.shape[0]
    filled = np.full(nnode, np.inf)
    filled[outlet] = z[outlet]
    done = np.zeros(nnode, bool)
    heap = [(z[outlet], outlet)]
    while heap:
        h, c = heapq.heappop(heap)
        if done[c]:
            continue
        done[c] = True
        for k in range(start[c], start[c + 1]):
            n = v[k]
            if done[n] or not interior[n]:
                continue
            fz = max(z[n], np.nextafter(h, np.inf) + 1e-6)
            if fz < filled[n]:
                filled[n] = fz
                heapq.heappush(heap, (fz, n))
    # steepest descent among graph nodes
    valid = np.isfinite(filled[u]) & np.isfinite(filled[v])
    dist = np.hypot(px[u] - px[v], py[u] - py[v])
    with np.errstate(invalid="ignore"):
        slope = np.where(valid, (filled[u] - filled[v]) / dist, -np.inf)
    down = -np.ones(nnode, np.int64)
    # per u: argmax slope (ties -> lowest v)
    order = np.lexsort((v, -slope, u))
    first = np.unique(u[order], return_index=True)
    cand_u = first[0]
    cand_k = order[first[1]]
    ok = (slope[cand_k] > 0.0) & interior[cand_u]
    down[cand_u[ok]] = v[cand_k[ok]]
    return down, filled


# ----------------------------------------------------------------------------
# reference initialisation formulas
# ----------------------------------------------------------------------------

def _river_eq_wid(order, depth, coeff):
    """RiverEqWid, src/init_river.c:99-124, with the C library's pow as the
    reference calls it (numpy's vectorised power can differ from it in the
    last bit, and differently on different processors)."""
    depth = np.maximum(depth, 0.0)
    out = np.where(order == RECTANGLE, coeff, 0.0)
    for k in np.nonzero(order != RECTANGLE)[0]:
        e = 1.0 / (float(order[k]) - 1.0)
        out[k] = 2.0 * math.pow(float(depth[k]) + RIVDPTHMIN, e) / math.pow(float(coeff[k]), e)
    return out


def generate(nelem: int = 1000, nriver: int = 100, seed: int = 0,
             length: float = 10000.0, shuffle: bool = True,
             shapes: str = "mixed", mesh: str = "grid") -> Watershed:
    """Build one synthetic watershed (reference order, 1-based ids).

    mesh: "grid" -- a jittered grid, two triangles per cell with the
    Delaunay diagonal (regular node degrees); "scattered" -- the Delaunay
    triangulation of scattered nodes (_scattered_points: irregular degrees
    and element sizes, as a mesh generator's output)."""
    rng = np.random.default_rng(seed)
    if mesh == "grid":
        nx, ny = _grid_shape(nelem)
        dx = length / (nx - 1)
        dy = length / (ny - 1)
        gi, gj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
        gi = gi.ravel()
        gj = gj.ravel()
        px = gi * dx
        py = gj * dy
        jx = rng.uniform(-0.3, 0.3, px.shape) * dx
        jy = rng.uniform(-0.3, 0.3, py.shape) * dy
        on_x_side = (gi == 0) | (gi == nx - 1)
        on_y_side = (gj == 0) | (gj == ny - 1)
        px = px + np.where(on_x_side, 0.0, jx)
        py = py + np.where(on_y_side, 0.0, jy)
        interior = ~(on_x_side | on_y_side)
        corner = on_x_side & on_y_side
    elif mesh == "scattered":
        px, py, interior, corner = _scattered_points(nelem, length, rng)
    else:
        raise ValueError(f"mesh must be 'grid' or 'scattered', not {mesh!r}")
    nnode = px.shape[0]

    hills = [(rng.uniform(0, length), rng.uniform(0, length),
              rng.uniform(20.0, 200.0), rng.uniform(500.0, 2000.0))
             for _ in range(8)]
    zmax_n = _dem(px, py, hills, length)
    dep_n = rng.uniform(2.0, 10.0, nnode)
    zmin_n = zmax_n - dep_n

    tri = _triangulate(nx, ny, px, py) if mesh == "grid" else _delaunay(px, py)
    ne = tri.shape[0]
    perm = rng.permutation(ne) if shuffle else np.arange(ne)
    tri = tri[perm]
    nb = _neighbours(tri)

    # ---- drainage network ----
    u, v, start = _node_adjacency(tri, nnode)
    has_interior_nb = np.zeros(nnode, bool)
    np.logical_or.at(has_interior_nb, u, interior[v])
    cand = np.where(~interior & has_interior_nb & ~corner)[0]
    outlet = int(cand[np.argmin(zmax_n[cand])])
    down_n, filled = _drainage(zmax_n, px, py, interior, outlet, u, v, start)
    in_graph = np.isfinite(filled)
    order = np.argsort(-filled[in_graph], kind="stable")
    nodes_desc = np.where(in_graph)[0][order]
    acc = np.ones(nnode)
    for n in nodes_desc:
        d = down_n[n]
        if d >= 0:
            acc[d] += acc[n]
    # keep the single network of the main stem: the interior node feeding the
    # outlet with the largest accumulation roots it
    feeders = np.where(interior & (down_n == outlet))[0]
    root = feeders[np.argmax(acc[feeders])]
    top = np.full(nnode, -1, np.int64)
    top[root] = root
    for n in nodes_desc[::-1]:
        d = down_n[n]
        if d >= 0 and top[d] >= 0 and interior[n]:
            top[n] = top[d]
    members = np.where(top == root)[0]
    rank = np.lexsort((members, -acc[members]))
    nr = min(nriver, members.shape[0])
    chosen = members[rank[:nr]]
    # reference order of segments: upstream (high filled elevation) first
    chosen = chosen[np.lexsort((chosen, -filled[chosen]))]
    seg_of_from = -np.ones(nnode, np.int64)
    seg_of_from[chosen] = np.arange(nr)
    from_n = chosen
    to_n = down_n[chosen]

    # left / right elements of every river edge (edge opposite node j of t)
    ea = np.concatenate([tri[:, 1], tri[:, 2], tri[:, 0]])
    eb = np.concatenate([tri[:, 2], tri[:, 0], tri[:, 1]])
    ew = np.concatenate([tri[:, 0], tri[:, 1], tri[:, 2]])
    et = np.tile(np.arange(ne), 3)
    ekey = np.minimum(ea, eb) * nnode + np.maximum(ea, eb)
    eord = np.argsort(ekey, kind="stable")
    eks = ekey[eord]
    rkey = np.minimum(from_n, to_n) * nnode + np.maximum(from_n, to_n)
    pos = np.searchsorted(eks, rkey)
    assert np.all(eks[pos + 1] == rkey), "river on a boundary edge"
    leftele = np.zeros(nr, np.int64)
    rightele = np.zeros(nr, np.int64)
    for off in (0, 1):
        k = eord[pos + off]
        t, w = et[k], ew[k]
        cr = ((px[to_n] - px[from_n]) * (py[w] - py[from_n])
              - (py[to_n] - py[from_n]) * (px[w] - px[from_n]))
        leftele = np.where(cr > 0.0, t + 1, leftele)
        rightele = np.where(cr > 0.0, rightele, t + 1)
    assert np.all(leftele > 0) and np.all(rightele > 0)
    down = np.where(seg_of_from[to_n] >= 0, seg_of_from[to_n] + 1, 0)

    # Stream burning: every river node lies at least 0.1 % of the segment
    # length below its upstream node.  The reference's channel routing moves
    # water upstream through a segment whose bed is above its upstream
    # neighbour's water surface even when that segment is empty
    # (ChanFlowRiverToRiver uses the upstream cross-section,
    # src/river_flow.c:257-300), so channels must fall downstream, as mesh
    # tools ensure by correcting river elevations (cf. CorrElev,
    # src/initialize.c:225-383).  Segments are visited upstream first.
    for s in range(nr):
        f, tn = int(from_n[s]), int(to_n[s])
        seglen = math.hypot(px[f] - px[tn], py[f] - py[tn])
        zcap = zmax_n[f] - 1e-3 * seglen
        if zmax_n[tn] > zcap:
            dz = zmax_n[tn] - zcap
            zmax_n[tn] -= dz
            zmin_n[tn] -= dz

    # ---- element geometry: InitTopo, src/init_topo.c:6-52 ----
    x = px[tri]
    y = py[tri]
    area = 0.5 * ((x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0])
                  - (y[:, 1] - y[:, 0]) * (x[:, 2] - x[:, 0]))
    assert np.all(area > 0.0)
    cx = (x[:, 0] + x[:, 1] + x[:, 2]) / 3.0
    cy = (y[:, 0] + y[:, 1] + y[:, 2]) / 3.0
    zmn = zmin_n[tri]
    zmx = zmax_n[tri]
    ezmin = (zmn[:, 0] + zmn[:, 1] + zmn[:, 2]) / 3.0
    ezmax = (zmx[:, 0] + zmx[:, 1] + zmx[:, 2]) / 3.0
    edge = np.empty((ne, 3))
    edge[:, 0] = np.sqrt((x[:, 1] - x[:, 2]) ** 2 + (y[:, 1] - y[:, 2]) ** 2)
    edge[:, 1] = np.sqrt((x[:, 2] - x[:, 0]) ** 2 + (y[:, 2] - y[:, 0]) ** 2)
    edge[:, 2] = np.sqrt((x[:, 0] - x[:, 1]) ** 2 + (y[:, 0] - y[:, 1]) ** 2)

    nabr = np.where(nb >= 0, nb + 1, 0).astype(np.int64)
    # river edges: src/init_river.c:23-33
    for s in range(nr):
        L, R = leftele[s] - 1, rightele[s] - 1
        for j in range(3):
            if nabr[L, j] == R + 1:
                nabr[L, j] = -(s + 1)
            if nabr[R, j] == L + 1:
                nabr[R, j] = -(s + 1)

    # ---- soil (per element) and land cover ----
    def logk():
        return np.power(10.0, np.clip(rng.normal(-5.0, 0.5, ne), -6.0, -4.0))
    ksath = logk()
    ksatv = logk()
    kinfv = ksatv * rng.uniform(1.0, 5.0, ne)
    porosity = rng.uniform(0.35, 0.5, ne)
    alpha = rng.uniform(0.5, 5.0, ne)
    beta = rng.uniform(1.2, 2.5, ne)
    depth = ezmax - ezmin
    dinf = np.full(ne, 0.1)
    dmac = np.minimum(rng.uniform(0.5, 2.0, ne), depth)
    areafh = rng.uniform(0.0, 0.1, ne)
    areafh[rng.uniform(size=ne) < 0.1] = 0.0
    areafv = rng.uniform(0.0, 0.1, ne)
    kmacv = 100.0 * kinfv
    kmach = 1000.0 * ksath
    rough = rng.uniform(0.03, 0.1, ne)
    rzd = rng.uniform(0.3, 2.0, ne)

    # ---- rivers: InitRiver, src/init_river.c:6-97 ----
    rx = 0.5 * (px[from_n] + px[to_n])
    ry = 0.5 * (py[from_n] + py[to_n])
    rzmax = 0.5 * (zmax_n[from_n] + zmax_n[to_n])
    L0, R0 = leftele - 1, rightele - 1
    rzmin = rzmax - (0.5 * (ezmax[L0] + ezmax[R0]) - 0.5 * (ezmin[L0] + ezmin[R0]))
    node_zmax = zmax_n[to_n]
    dist_left = np.sqrt((rx - cx[L0]) * (rx - cx[L0]) + (ry - cy[L0]) * (ry - cy[L0]))
    dist_right = np.sqrt((rx - cx[R0]) * (rx - cx[R0]) + (ry - cy[R0]) * (ry - cy[R0]))
    accn = acc[from_n] / acc[from_n].max()
    rdepth = 0.5 + 1.5 * np.power(accn, 0.3)
    if shapes == "mixed":
        u01 = rng.uniform(size=nr)
        order_r = np.where(u01 < 0.55, RECTANGLE,
                           np.where(u01 < 0.7, TRIANGLE,
                                    np.where(u01 < 0.85, QUADRATIC, CUBIC)))
    else:
        order_r = np.full(nr, RECTANGLE)
    wtarget = 2.0 + 18.0 * np.sqrt(accn)
    dm = rdepth + RIVDPTHMIN
    coeff = np.where(order_r == RECTANGLE, wtarget,
                     np.where(order_r == TRIANGLE, 2.0 * dm / wtarget,
                              np.where(order_r == QUADRATIC, 4.0 * dm / wtarget ** 2,
                                       8.0 * dm / wtarget ** 3)))
    rlength = np.sqrt((px[from_n] - px[to_n]) ** 2 + (py[from_n] - py[to_n]) ** 2)
    rwidth = _river_eq_wid(order_r, rdepth, coeff)
    rzbed = rzmax - rdepth
    rrough = rng.uniform(0.03, 0.06, nr)
    rcwr = np.full(nr, 0.6)
    rksath = np.power(10.0, rng.uniform(-5.0, -4.3, nr))
    rksatv = np.power(10.0, rng.uniform(-5.5, -4.5, nr))
    rbed = rng.uniform(0.1, 1.0, nr)
    rpor = 0.5 * (porosity[L0] + porosity[R0])
    rarea = rlength * _river_eq_wid(order_r, rdepth, coeff)
    out_seg = np.where(down == 0)[0]
    for s in out_seg:
        f, tn = from_n[s], to_n[s]
        down[s] = ZERO_DPTH_GRAD if zmax_n[f] > zmax_n[tn] else CRIT_DPTH

    # ---- neighbour centroids / distances: InitSurfL, src/initialize.c:385-458
    nabr_x = np.empty((ne, 3))
    nabr_y = np.empty((ne, 3))
    nabrdist = np.empty((ne, 3))
    mids = [(1, 2), (2, 0), (0, 1)]
    circ = edge[:, 0] * edge[:, 1] * edge[:, 2] / (4.0 * area)
    for j, (a, b) in enumerate(mids):
        distx = cx - 0.5 * (x[:, a] + x[:, b])
        disty = cy - 0.5 * (y[:, a] + y[:, b])
        nj = nabr[:, j]
        bnd = nj == 0
        ele = nj > 0
        riv = nj < 0
        nabr_x[bnd, j] = cx[bnd] - 2.0 * distx[bnd]
        nabr_y[bnd, j] = cy[bnd] - 2.0 * disty[bnd]
        nabrdist[bnd, j] = np.sqrt(circ[bnd] ** 2 - (edge[bnd, j] / 2.0) ** 2)
        nabr_x[ele, j] = cx[nj[ele] - 1]
        nabr_y[ele, j] = cy[nj[ele] - 1]
        nabr_x[riv, j] = rx[-nj[riv] - 1]
        nabr_y[riv, j] = ry[-nj[riv] - 1]
        m = ~bnd
        d2 = (cx[m] - nabr_x[m, j]) * (cx[m] - nabr_x[m, j])
        d2 = d2 + (cy[m] - nabr_y[m, j]) * (cy[m] - nabr_y[m, j])
        nabrdist[m, j] = np.sqrt(d2)

    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    f64 = lambda a: np.ascontiguousarray(a, np.float64)
    arrays = {
        "nabr": i32(nabr), "bc_type": i32(np.zeros((ne, 3))),
        "area": f64(area), "zmin": f64(ezmin), "zmax": f64(ezmax),
        "edge": f64(edge), "nabrdist": f64(nabrdist), "nabr_x": f64(nabr_x),
        "nabr_y": f64(nabr_y), "depth": f64(depth), "ksath": f64(ksath),
        "ksatv": f64(ksatv), "kinfv": f64(kinfv), "dinf": f64(dinf),
        "alpha": f64(alpha), "beta": f64(beta), "porosity": f64(porosity),
        "dmac": f64(dmac), "kmach": f64(kmach), "kmacv": f64(kmacv),
        "areafv": f64(areafv), "areafh": f64(areafh), "rough": f64(rough),
        "rzd": f64(rzd),
        "down": i32(down), "leftele": i32(leftele), "rightele": i32(rightele),
        "intrpl_ord": i32(order_r), "riverbc_type": i32(np.zeros(nr)),
        "riv_area": f64(rarea), "riv_zmin": f64(rzmin), "riv_zmax": f64(rzmax),
        "riv_zbed": f64(rzbed), "riv_node_zmax": f64(node_zmax),
        "riv_dist_left": f64(dist_left), "riv_dist_right": f64(dist_right),
        "riv_depth": f64(rdepth), "riv_coeff": f64(coeff),
        "riv_length": f64(rlength), "riv_width": f64(rwidth),
        "riv_rough": f64(rrough), "riv_cwr": f64(rcwr),
        "riv_ksath": f64(rksath), "riv_ksatv": f64(rksatv),
        "riv_bedthick": f64(rbed), "riv_porosity": f64(rpor),
    }
    nodes = {"x": px, "y": py, "zmin": zmin_n, "zmax": zmax_n, "tri": tri,
             "from_n": np.asarray(from_n), "to_n": np.asarray(to_n)}
    return Watershed(ne, nr, arrays, seed=seed, x=cx, y=cy, nodes=nodes)


# ----------------------------------------------------------------------------
# states and forcing
# ----------------------------------------------------------------------------

def relax_state(ws: Watershed) -> np.ndarray:
    """RelaxIc initial condition (src/initialize.c:496-575): surf 0,
    unsat 0.1 m, gw = depth - 0.1, stage 0, river gw = zbed - zmin - 0.1."""
    a = ws.arrays
    y = np.zeros(ws.neq)
    ne, nr = ws.nelem, ws.nriver
    y[ne:2 * ne] = 0.1
    y[2 * ne:3 * ne] = a["depth"] - 0.1
    y[3 * ne + nr:] = a["riv_zbed"] - a["riv_zmin"] - 0.1
    return y


def reference_state(ws: Watershed, seed: int = 1) -> np.ndarray:
    """A wet mid-event state that reaches every branch of the right-hand side:
    dry / shallow / ponded surfaces, unsaturated and saturated columns,
    empty to overtopped channels."""
    rng = np.random.default_rng(seed)
    a = ws.arrays
    ne, nr = ws.nelem, ws.nriver
    depth = a["depth"]
    y = np.zeros(ws.neq)
    gw = depth * rng.uniform(0.2, 0.95, ne)
    sat = rng.uniform(size=ne) < 0.1
    gw[sat] = depth[sat] - a["dinf"][sat] * rng.uniform(0.0, 0.9, sat.sum())
    deficit = depth - gw
    unsat = deficit * rng.uniform(0.05, 0.98, ne)
    cls = rng.uniform(size=ne)
    surf = np.where(cls < 0.35, 0.0,
                    np.where(cls < 0.55, rng.uniform(0.0, 0.5 * DEPRSTG, ne),
                             rng.uniform(DEPRSTG, 0.05, ne)))
    y[:ne] = surf
    y[ne:2 * ne] = unsat
    y[2 * ne:3 * ne] = gw
    rd = a["riv_depth"]
    y[3 * ne:3 * ne + nr] = rd * rng.uniform(0.05, 1.5, nr)
    y[3 * ne + nr:] = (a["riv_zbed"] - a["riv_zmin"]) * rng.uniform(0.5, 1.05, nr)
    return y


def jitter(y: np.ndarray, seed: int, lo: float = 0.9, hi: float = 1.1) -> np.ndarray:
    """A storage-wise jitter of a state, x U(lo, hi)."""
    rng = np.random.default_rng(seed)
    return y * rng.uniform(lo, hi, y.shape)


def hourly_forcing(ws: Watershed, hours: int, seed: int = 2):
    """Hourly precipitation (Bernoulli(0.1) wet hours, gamma(k=0.7,
    theta=3 mm/h) amounts) and PET (0.3 mm/h * max(0, sin(2 pi (h-6)/24))),
    uniform over the domain.  ET is split by a fixed rule: edir = 0.3 PET,
    ett = 0.7 PET; pcpdrp = precipitation.  Returns three [hours] arrays in
    m/s."""
    rng = np.random.default_rng(seed)
    wet = rng.uniform(size=hours) < 0.1
    amount = rng.gamma(0.7, 3.0, hours)
    prcp = np.where(wet, amount, 0.0) / 3.6e6
    h = np.arange(hours)
    pet = 0.3 * np.maximum(0.0, np.sin(2.0 * np.pi * (h - 6) / 24.0)) / 3.6e6
    return prcp, 0.3 * pet, 0.7 * pet


def random_forcing(ws: Watershed, seed: int = 3):
    """Per-element forcing for single-call parity cases (m/s)."""
    rng = np.random.default_rng(seed)
    ne = ws.nelem
    pcpdrp = np.where(rng.uniform(size=ne) < 0.5, rng.gamma(0.7, 3.0, ne), 0.0) / 3.6e6
    pet = rng.uniform(0.0, 0.3, ne) / 3.6e6
    return pcpdrp, 0.3 * pet, 0.7 * pet


def noah_inputs(ws: Watershed, seed: int = 4, nlayers: int = 4) -> dict:
    """Synthetic per-step outputs of the Noah land-surface model that the
    Flux-PIHM right-hand side reads: transpiration per soil layer et
    [nelem, nlayers] (m/s), the water-table layer nwtbl (0..nlayers+1) and the
    root layers nroot (1..nlayers), the top layer's unfrozen moisture sh2o0
    between the residual and saturated contents smcmin / smcmax (a few outside
    to reach the saturation clamps; smcmax - smcmin = porosity), and the
    frozen-soil infiltration factor fcr (1 for unfrozen soil, 0.3..1 for
    a third of the elements)."""
    rng = np.random.default_rng(9000 + seed)
    ne = ws.nelem
    por = ws.arrays["porosity"]
    smcmin = rng.uniform(0.02, 0.08, ne)
    smcmax = smcmin + por
    et = rng.uniform(0.0, 2e-8, (ne, nlayers)) * (rng.random((ne, nlayers)) < 0.8)
    nwtbl = rng.integers(0, nlayers + 2, ne).astype(np.int32)
    nroot = rng.integers(1, nlayers + 1, ne).astype(np.int32)
    sh2o0 = smcmin + por * rng.uniform(-0.05, 1.05, ne)
    fcr = np.where(rng.random(ne) < 1.0 / 3.0, rng.uniform(0.3, 1.0, ne), 1.0)
    return dict(et=et, nwtbl=nwtbl, nroot=nroot, sh2o0=sh2o0, smcmin=smcmin, smcmax=smcmax, fcr=fcr)
