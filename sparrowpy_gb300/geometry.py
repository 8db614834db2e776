"""Host-side scene description: polygons, wall patching, direction frames.

These are the inputs of the GPU path: the reference builds them in Python as
well (sparrowpy/geometry.py, sparrowpy/testing/stub_utils.py,
sparrowpy/classes/RadiosityFast.py:971-986).  They run once per scene, not
per solve.
"""
import numpy as np

from .coords import Coordinates, _cart
from .sound_object import Receiver, SoundSource  # noqa: F401  (sparrowpy/geometry.py:12 re-exports them)


def _norm(v):
    v = np.asarray(v, dtype=float)
    return v / np.sqrt(np.dot(v, v))


class Polygon:
    """Planar polygon: points (n_points, 3), up vector and normal.

    Mirrors sparrowpy/geometry.py:15-62 (checks: >= 3 points, coplanar
    points, normal perpendicular to the plane).
    """

    def __init__(self, points, up_vector, normal):
        self.pts = np.array(points, dtype=float)
        normal = np.array(normal, dtype=float)
        assert self.pts.shape[1] >= 3, 'You need at least 3 points to build a Polygon'
        if self.pts.shape[0] > 3:
            x_0 = self.pts[0]
            for i in range(1, self.pts.shape[0] - 2):
                det = np.linalg.det([x_0 - self.pts[i], x_0 - self.pts[i + 1], x_0 - self.pts[i + 2]])
                assert abs(det) < 1e-10, 'Points must be in a plane to create a Polygon'
        self.up_vector = _norm(up_vector)
        calc_normal = _norm(np.cross(self.pts[0] - self.pts[1], self.pts[0] - self.pts[2]))
        assert all(np.abs(np.cross(normal, calc_normal)) < 1e-10), \
            'The normal vector is not perpendicular to the polygon'
        self._normal = normal

    @property
    def normal(self):
        return self._normal

    @property
    def n_points(self):
        return self.pts.shape[0]

    @property
    def center(self):
        return np.sum(self.pts, axis=0) / self.pts.shape[0]

    @property
    def size(self):
        """Extent (l, m, n) as the reference computes it: |(p0 - p1) - (p1 - p2)| (geometry.py:84-89)."""
        return np.abs((self.pts[0] - self.pts[1]) - (self.pts[1] - self.pts[2]))

    @property
    def area(self):
        """Area in m^2 (geometry.py:91-121): one triangle, two triangles (0, 1, 2) and (2, 3, 0), or for more
        points the fan of triangles (p_i, p_i+1, centre)."""
        pts = self.pts
        if len(pts) == 3:
            tris = np.array([pts])
        elif len(pts) == 4:
            tris = np.array([pts[0:3], [pts[2], pts[3], pts[0]]])
        else:
            c = self.center
            tris = np.array([[pts[i % len(pts)], pts[(i + 1) % len(pts)], c] for i in range(len(pts))])
        area = 0
        for tri in tris:
            area += .5 * np.linalg.norm(np.cross(tri[1] - tri[0], tri[2] - tri[0]))
        return area

    def on_surface(self, point):
        """True if the point lies on the polygon: the angles its vertices subtend sum to 2 pi, or it is a
        vertex (geometry.py:132-153, absolute tolerance 1e-12)."""
        n = self.pts.shape[0]
        p = np.asarray(point, dtype=float)
        sum_angle = 0
        for i in range(n):
            v1 = self.pts[i] - p
            v2 = self.pts[(i + 1) % n] - p
            m1, m2 = np.sqrt(np.dot(v1, v1)), np.sqrt(np.dot(v2, v2))
            if abs(m1 * m2) < 1e-12:
                return True
            sum_angle = sum_angle + np.arccos(np.dot(v1, v2) / (m1 * m2))
        return abs(sum_angle - 2 * np.pi) < 1e-12

    def intersection(self, origin, direction):
        """Intersection of the ray origin + t direction (t > 0) with the polygon, or None
        (geometry.py:155-193)."""
        origin = np.asarray(origin, dtype=float)
        direction = np.asarray(direction, dtype=float)
        n = self.normal
        if abs(np.dot(direction, n)) < 1e-12:
            return None
        t = 1 / (np.dot(direction, n)) * (np.dot(n, self.pts[0]) - np.dot(n, origin))
        if t <= 0.0:
            return None
        point = origin + t * direction
        return point if self.on_surface(point) else None

    def to_dict(self):
        return {'up_vector': self.up_vector.tolist(), 'pts': self.pts.tolist(), 'normal': self._normal.tolist()}

    @classmethod
    def from_dict(cls, d):
        return cls(d['pts'], d['up_vector'], d['normal'])


class _Environment:
    """Walls, a source, a receiver and the speed of sound (geometry.py:232-273, without plotting)."""

    def __init__(self, polygons, source, receiver, speed_of_sound):
        self.speed_of_sound = speed_of_sound
        self.polygons = polygons
        self.source = source
        self.receiver = receiver


def shoebox_room_stub(length_x, length_y, length_z):
    """Six inward-facing walls of a shoebox (sparrowpy/testing/stub_utils.py:5-48)."""
    lx, ly, lz = length_x, length_y, length_z
    return [
        Polygon([[0, 0, 0], [lx, 0, 0], [lx, 0, lz], [0, 0, lz]], [1, 0, 0], [0, 1, 0]),
        Polygon([[0, ly, 0], [lx, ly, 0], [lx, ly, lz], [0, ly, lz]], [1, 0, 0], [0, -1, 0]),
        Polygon([[0, 0, 0], [lx, 0, 0], [lx, ly, 0], [0, ly, 0]], [1, 0, 0], [0, 0, 1]),
        Polygon([[0, 0, lz], [lx, 0, lz], [lx, ly, lz], [0, ly, lz]], [1, 0, 0], [0, 0, -1]),
        Polygon([[0, 0, 0], [0, 0, lz], [0, ly, lz], [0, ly, 0]], [0, 0, 1], [1, 0, 0]),
        Polygon([[lx, 0, 0], [lx, 0, lz], [lx, ly, lz], [lx, ly, 0]], [0, 0, 1], [-1, 0, 0]),
    ]


def _patch_axes(polygon_points, max_size):
    size = polygon_points.max(axis=0) - polygon_points.min(axis=0)
    patch_nums = np.array([int(n) for n in size / max_size])
    x_idx = y_idx = None
    if patch_nums[2] == 0:
        x_idx, y_idx = 0, 1
    if patch_nums[1] == 0:
        x_idx, y_idx = 0, 2
    if patch_nums[0] == 0:
        x_idx, y_idx = 1, 2
    if x_idx is None:
        raise ValueError("only axis-aligned rectangular walls can be patched")
    return size, patch_nums, x_idx, y_idx


def total_number_of_patches(polygon_points, max_size):
    """sparrowpy/geometry.py:341-371 `_total_number_of_patches`."""
    _, patch_nums, x_idx, y_idx = _patch_axes(np.asarray(polygon_points, float), max_size)
    return int(patch_nums[x_idx] * patch_nums[y_idx])


def create_patches(polygon_points, max_size):
    """sparrowpy/geometry.py:373-410 `_create_patches` (axis-aligned walls)."""
    polygon_points = np.asarray(polygon_points, dtype=float)
    size, patch_nums, x_idx, y_idx = _patch_axes(polygon_points, max_size)
    with np.errstate(divide='ignore', invalid='ignore'):
        real_size = size / patch_nums
    x_min = np.min(polygon_points.T[x_idx])
    y_min = np.min(polygon_points.T[y_idx])
    n = int(patch_nums[x_idx] * patch_nums[y_idx])
    out = np.empty((n, 4, 3))
    i = 0
    for i_x in range(patch_nums[x_idx]):
        for i_y in range(patch_nums[y_idx]):
            points = polygon_points.copy()
            points[0, x_idx] = x_min + i_x * real_size[x_idx]
            points[0, y_idx] = y_min + i_y * real_size[y_idx]
            points[1, x_idx] = x_min + (i_x + 1) * real_size[x_idx]
            points[1, y_idx] = y_min + i_y * real_size[y_idx]
            points[3, x_idx] = x_min + i_x * real_size[x_idx]
            points[3, y_idx] = y_min + (i_y + 1) * real_size[y_idx]
            points[2, x_idx] = x_min + (i_x + 1) * real_size[x_idx]
            points[2, y_idx] = y_min + (i_y + 1) * real_size[y_idx]
            out[i] = points
            i += 1
    return out


def axis_patchable(polygon_points, max_size):
    """True where the reference's patching applies: some axis spans less than max_size."""
    size = np.ptp(np.asarray(polygon_points, dtype=float), axis=0)
    return bool(np.any(np.array([int(n) for n in size / max_size]) == 0))


def create_patches_general(polygon_points, max_size):
    """Patches of a planar convex quadrilateral wall in any orientation.

    The reference patches walls that are aligned with the coordinate axes
    (geometry.py:373-410) and fails on others.  Here the wall is split along
    its own edges p0 -> p1 (u) and p0 -> p3 (v) into n_u x n_v
    quadrilaterals, n = max(1, int(edge length / max_size)) as the reference
    counts patches per axis.  Corners are bilinear in (u, v) and keep the
    wall's vertex order; u runs in the outer loop, v in the inner, as the
    reference's loops do.
    """
    p = np.asarray(polygon_points, dtype=float)
    if p.shape != (4, 3):
        raise ValueError("general patching takes quadrilateral walls (4 vertices)")
    n = np.cross(p[1] - p[0], p[3] - p[0])
    nn = np.sqrt(np.sum(n * n))
    extent = float(np.max(np.ptp(p, axis=0)))
    if nn <= 1e-12 * max(extent, 1.0) ** 2:
        raise ValueError("degenerate wall")
    n = n / nn
    if np.max(np.abs((p - p[0]) @ n)) > 1e-9 * max(extent, 1.0):
        raise ValueError("the wall's vertices are not coplanar")
    for k in range(4):
        turn = np.cross(p[(k + 1) % 4] - p[k], p[(k + 2) % 4] - p[(k + 1) % 4]) @ n
        if turn <= 0:
            raise ValueError("the wall is not a convex quadrilateral")
    # 1e-6 of a patch absorbs the rounding of rotated coordinates (also of
    # float32 ones, as STL files store them), so that an edge of k patch
    # sizes gives k patches as on an axis-aligned wall
    n_u = max(1, int(np.sqrt(np.sum((p[1] - p[0]) ** 2)) / max_size + 1e-6))
    n_v = max(1, int(np.sqrt(np.sum((p[3] - p[0]) ** 2)) / max_size + 1e-6))

    def at(s, t):
        return (1 - s) * (1 - t) * p[0] + s * (1 - t) * p[1] + s * t * p[2] + (1 - s) * t * p[3]

    out = np.empty((n_u * n_v, 4, 3))
    k = 0
    for a in range(n_u):
        for b in range(n_v):
            s0, s1, t0, t1 = a / n_u, (a + 1) / n_u, b / n_v, (b + 1) / n_v
            out[k] = (at(s0, t0), at(s1, t0), at(s1, t1), at(s0, t1))
            k += 1
    return out


def create_patches_triangles(polygon_points, max_size):
    """Triangular patches of a planar convex polygon wall of 3 or more vertices (no counterpart in the reference).

    The wall is cut into the fan (p0, p_k, p_k+1), k = 1 .. nv - 2; each
    triangle (a, b, c) into n x n similar triangles, n = max(1, int(longest
    side / max_size)), with corners a + (i/n)(b - a) + (j/n)(c - a).  Every
    patch keeps the wall's vertex order, so its normal is the wall's.  The
    form factors, visibility and point factors take triangles as the
    reference's universal method defines them (universal.py:12-96,
    integration.py:533-605 with its triangle branch).
    """
    p = np.asarray(polygon_points, dtype=float)
    if p.ndim != 2 or p.shape[0] < 3 or p.shape[1] != 3:
        raise ValueError("a wall needs at least 3 vertices")
    out = []
    for k in range(1, p.shape[0] - 1):
        a, b, c = p[0], p[k], p[k + 1]
        longest = max(np.sqrt(np.sum((b - a) ** 2)), np.sqrt(np.sum((c - b) ** 2)), np.sqrt(np.sum((a - c) ** 2)))
        n = max(1, int(longest / max_size + 1e-6))

        def at(i, j):
            return a + (i / n) * (b - a) + (j / n) * (c - a)

        for i in range(n):
            for j in range(n - i):
                out.append((at(i, j), at(i + 1, j), at(i, j + 1)))
                if i + j < n - 1:
                    out.append((at(i + 1, j), at(i + 1, j + 1), at(i, j + 1)))
    return np.array(out, dtype=float).reshape(-1, 3, 3)


def process_patches(walls_points, walls_normal, patch_size):
    """sparrowpy/geometry.py:290-339 `_process_patches`.

    Quadrilateral walls: axis-aligned ones are patched as the reference
    does, with its arithmetic; any other (where the reference fails) by
    create_patches_general; the patches are quadrilaterals.  Walls of any
    other vertex count (all walls share one, as the arrays demand):
    triangular patches (create_patches_triangles).  Returns patches_points
    (n, 4 or 3, 3), patches_normal (n, 3), n_patches and patch_to_wall_ids
    (n,).
    """
    walls_points = np.asarray(walls_points, dtype=float)
    if walls_points.ndim == 3 and walls_points.shape[1] != 4:
        parts = [create_patches_triangles(w, patch_size) for w in walls_points]
        nv = 3
    else:
        parts = [create_patches(w, patch_size) if axis_patchable(w, patch_size)
                 else create_patches_general(w, patch_size) for w in walls_points]
        nv = 4
    patches_points = np.concatenate(parts, axis=0) if parts else np.zeros((0, nv, 3))
    patch_to_wall_ids = np.concatenate(
        [np.full(p.shape[0], i, dtype=np.int64) for i, p in enumerate(parts)]) if parts else np.zeros(0, np.int64)
    patches_normal = np.asarray(walls_normal, dtype=float)[patch_to_wall_ids, :]
    return patches_points, patches_normal, patches_points.shape[0], patch_to_wall_ids


def calculate_center(points):
    """sparrowpy/geometry.py:412-413 (host copy used by the properties)."""
    points = np.asarray(points, dtype=float)
    return np.sum(points, axis=-2) / points.shape[-2]


def calculate_size(points):
    """sparrowpy/geometry.py:415-418."""
    points = np.asarray(points, dtype=float)
    vec1 = points[..., 0, :] - points[..., 1, :]
    vec2 = points[..., 1, :] - points[..., 2, :]
    return np.abs(vec1 - vec2)


def calculate_area(points):
    """sparrowpy/geometry.py:420-448 (fan triangulation, host copy)."""
    points = np.asarray(points, dtype=float)
    area = np.zeros(points.shape[0])
    for t in range(points.shape[1] - 2):
        c = np.cross(points[:, t + 1] - points[:, 0], points[:, t + 2] - points[:, 0])
        area += .5 * np.sqrt(np.sum(c * c, axis=-1))
    return area


def wall_frame(normal, up_vector):
    """Rotation taking the BRDF frame (normal +z, up +x) to a wall's frame.

    RadiosityFast.py:971-986 builds it from two pyfar orientations
    (view/up); the result maps local z to the wall normal, local x to the
    up vector and local y to normal x up.  Columns: (up, n x up, n).
    """
    n = _norm(normal)
    up = _norm(up_vector)
    return np.stack([up, np.cross(n, up), n], axis=1)


def rotate_coords_to_normal(wall_normal, wall_up_vector, sources, receivers):
    """RadiosityFast.py:971-986 `_rotate_coords_to_normal`.

    Rotates both direction sets into the wall frame and normalises them to
    radius 1.  Returns Coordinates copies (weights kept).
    """
    rot = wall_frame(wall_normal, wall_up_vector)
    out = []
    for c in (sources, receivers):
        xyz = _cart(c).reshape(-1, 3) @ rot.T
        xyz = xyz / np.sqrt(np.sum(xyz * xyz, axis=-1))[:, None]
        w = getattr(c, "weights", None)
        out.append(Coordinates.from_cartesian(xyz, weights=None if w is None else np.asarray(w).reshape(-1)))
    return out[0], out[1]
