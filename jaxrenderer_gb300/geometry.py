"""Camera and matrix math of the rasteriser, on the host.

Mirrors renderer/geometry.py of jaxrenderer: the Camera NamedTuple and its
constructors (view, perspective, orthographic, viewport matrices), the
point/vector transforms and the quaternion helpers.  These are per-scene 4x4
set-up computations; they run once per call in NumPy with the reference's
FP32 operation order (products summed in index order, one rounding per
operation).  `dtype=np.float64` gives the double twin used by the
finite-difference gradient checks.
"""
from __future__ import annotations

import enum
from typing import NamedTuple

import numpy as np

F32 = np.float32


def _arr(x, dtype=None) -> np.ndarray:
    if hasattr(x, "detach"):  # torch tensor
        x = x.detach().cpu().numpy()
    a = np.asarray(x)
    if dtype is not None:
        a = a.astype(dtype, copy=False)
    elif not np.issubdtype(a.dtype, np.floating):
        a = a.astype(F32)
    return a


def matmul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """(..., n, k) @ (k, m) with products summed in index order."""
    a = np.asarray(a)
    b = np.asarray(b)
    dt = np.result_type(a, b)
    a = a.astype(dt, copy=False)
    b = b.astype(dt, copy=False)
    acc = a[..., :, 0:1] * b[0:1, :]
    for k in range(1, a.shape[-1]):
        acc = acc + a[..., :, k : k + 1] * b[k : k + 1, :]
    return acc


def matvec(m: np.ndarray, v: np.ndarray) -> np.ndarray:
    """out[..., i] = sum_k v[..., k] * m[i, k], index order (Camera.apply)."""
    m = np.asarray(m)
    v = np.asarray(v)
    dt = np.result_type(m, v)
    acc = v[..., 0:1].astype(dt) * m[:, 0].astype(dt)
    for k in range(1, v.shape[-1]):
        acc = acc + v[..., k : k + 1].astype(dt) * m[:, k].astype(dt)
    return acc


def _sum_sq(v: np.ndarray) -> np.ndarray:
    """Sum of squares of every element, accumulated sequentially in index
    order (the order the device-side merge uses for the same global norms)."""
    flat = v.reshape(-1)
    if flat.size <= 4:
        acc = flat[0] * flat[0]
        for k in range(1, flat.size):
            acc = acc + flat[k] * flat[k]
        return acc
    return np.add.accumulate(flat * flat, dtype=v.dtype)[-1]


def normalise(vector) -> np.ndarray:
    """vector / jnp.linalg.norm(vector) (geometry.py:39-47).

    The norm is taken over every element: for an (N, 3) batch this is one
    global norm, as in the reference.
    """
    v = _arr(vector)
    return v / np.sqrt(_sum_sq(v))


class Interpolation(enum.Enum):
    """Interpolation qualifiers (geometry.py:50-110)."""

    FLAT = 0
    NOPERSPECTIVE = 1
    SMOOTH = 2

    def __call__(self, values, barycentric_screen, barycentric_clip):
        values = _arr(values)
        if self == Interpolation.FLAT:
            coef = np.array([1, 0, 0], dtype=values.dtype)
        elif self == Interpolation.NOPERSPECTIVE:
            coef = _arr(barycentric_screen)
        else:
            coef = _arr(barycentric_clip)
        acc = coef[0] * values[0]
        for k in range(1, 3):
            acc = acc + coef[k] * values[k]
        return acc


def interpolate(values, barycentric_screen, barycentric_clip, mode=Interpolation.SMOOTH):
    """Convenience wrapper of Interpolation.__call__ (geometry.py:120-138)."""
    return mode(values, barycentric_screen, barycentric_clip)


def to_homogeneous(coordinates, value=1.0) -> np.ndarray:
    """Append `value` on the last axis (geometry.py:144-163)."""
    c = _arr(coordinates)
    pad = np.broadcast_to(np.asarray(value, dtype=c.dtype), c.shape[:-1] + (1,))
    return np.concatenate([c, pad], axis=-1)


def normalise_homogeneous(coordinates) -> np.ndarray:
    """Divide by the last component (geometry.py:169-179)."""
    c = _arr(coordinates)
    return c / c[..., -1:]


def to_cartesian(coordinates) -> np.ndarray:
    """Divide by w (keep as is where w == 0) and drop it (geometry.py:185-202)."""
    c = _arr(coordinates)
    w = c[..., -1:]
    with np.errstate(divide="ignore", invalid="ignore"):
        div = c / w
    return np.where(w == 0.0, c[..., :-1], div[..., :-1])


def cross(a, b) -> np.ndarray:
    a = _arr(a)
    b = _arr(b)
    return np.stack(
        [
            a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
            a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
            a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0],
        ],
        axis=-1,
    )


def lu_inverse(m) -> np.ndarray:
    """jnp.linalg.inv of a batch of n x n matrices: LU with partial pivoting
    (reference LAPACK getf2 order) and two triangular solves (reference BLAS
    trsm order), vectorised over the leading axes."""
    a = _arr(m).copy()
    dt = a.dtype
    n = a.shape[-1]
    batch = a.shape[:-2]
    a = a.reshape((-1, n, n))
    nb = a.shape[0]
    rows = np.arange(nb)
    perm = np.tile(np.arange(n), (nb, 1))
    tiny = np.finfo(dt).tiny
    for j in range(n - 1):
        col = np.abs(a[:, j:, j])
        # first index of the maximum (NaN never wins, as with `>`)
        p = np.zeros(nb, dtype=np.int64)
        best = col[:, 0].copy()
        for r in range(1, n - j):
            better = col[:, r] > best
            p = np.where(better, r, p)
            best = np.where(better, col[:, r], best)
        p = p + j
        nz = a[rows, p, j] != 0
        swap = nz & (p != j)
        if np.any(swap):
            idx = rows[swap]
            rj = a[idx, j, :].copy()
            a[idx, j, :] = a[idx, p[swap], :]
            a[idx, p[swap], :] = rj
            pj = perm[idx, j].copy()
            perm[idx, j] = perm[idx, p[swap]]
            perm[idx, p[swap]] = pj
        piv = a[:, j, j]
        normal = nz & (np.abs(piv) >= tiny)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            rcp = (np.asarray(1, dtype=dt) / piv).astype(dt)
            for r in range(j + 1, n):
                scaled = np.where(normal, a[:, r, j] * rcp, a[:, r, j] / piv)
                a[:, r, j] = np.where(nz, scaled, a[:, r, j])
            for r in range(j + 1, n):
                for c in range(j + 1, n):
                    a[:, r, c] = a[:, r, c] - a[:, r, j] * a[:, j, c]
    out = np.zeros_like(a)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for colidx in range(n):
            b = (perm == colidx).astype(dt)
            for k in range(n):
                nzk = b[:, k] != 0
                for i in range(k + 1, n):
                    b[:, i] = np.where(nzk, b[:, i] - b[:, k] * a[:, i, k], b[:, i])
            for k in range(n - 1, -1, -1):
                nzk = b[:, k] != 0
                bk = np.where(nzk, b[:, k] / a[:, k, k], b[:, k])
                b[:, k] = bk
                for i in range(k):
                    b[:, i] = np.where(nzk, b[:, i] - bk * a[:, i, k], b[:, i])
            out[:, :, colidx] = b
    return out.reshape(batch + (n, n))


def det3(m) -> np.ndarray:
    """jnp.linalg.det closed form for 3x3 matrices, left to right."""
    a = _arr(m)
    t1 = (a[..., 0, 0] * a[..., 1, 1]) * a[..., 2, 2]
    t2 = (a[..., 0, 1] * a[..., 1, 2]) * a[..., 2, 0]
    t3 = (a[..., 0, 2] * a[..., 1, 0]) * a[..., 2, 1]
    t4 = (a[..., 0, 2] * a[..., 1, 1]) * a[..., 2, 0]
    t5 = (a[..., 0, 0] * a[..., 1, 2]) * a[..., 2, 1]
    t6 = (a[..., 0, 1] * a[..., 1, 0]) * a[..., 2, 2]
    return ((((t1 + t2) + t3) - t4) - t5) - t6


# ------------------------------------------- batched (leading axis) twins
#
# Per-scene set-up of many cameras at once.  Each function gives, for every
# index of the leading axis, the bits its single-camera counterpart gives:
# the same operations in the same order, applied elementwise.


def normalise_rows(v) -> np.ndarray:
    """normalise() of every 3-vector along the last axis (one norm per row,
    sum of squares in index order)."""
    v = _arr(v)
    return v / np.sqrt((v[..., 0:1] * v[..., 0:1] + v[..., 1:2] * v[..., 1:2]) + v[..., 2:3] * v[..., 2:3])


def bmatmul(a, b) -> np.ndarray:
    """(..., n, k) @ (..., k, m) with products summed in index order."""
    a = np.asarray(a)
    b = np.asarray(b)
    dt = np.result_type(a, b)
    a = a.astype(dt, copy=False)
    b = b.astype(dt, copy=False)
    acc = a[..., :, 0:1] * b[..., 0:1, :]
    for k in range(1, a.shape[-1]):
        acc = acc + a[..., :, k : k + 1] * b[..., k : k + 1, :]
    return acc


def bmatvec(m, v) -> np.ndarray:
    """out[..., i] = sum_k v[..., k] * m[..., i, k] in index order (Camera.apply
    with one matrix per leading index)."""
    m = np.asarray(m)
    v = np.asarray(v)
    dt = np.result_type(m, v)
    acc = v[..., None, 0].astype(dt) * m[..., :, 0].astype(dt)
    for k in range(1, v.shape[-1]):
        acc = acc + v[..., None, k].astype(dt) * m[..., :, k].astype(dt)
    return acc


def _look_at_rows(eye, centre, up):
    eye = _arr(eye)
    centre = np.broadcast_to(_arr(centre, eye.dtype), eye.shape)
    up = np.broadcast_to(_arr(up, eye.dtype), eye.shape)
    forward = normalise_rows(centre - eye)
    up = normalise_rows(up)
    side = normalise_rows(cross(forward, up))
    up = cross(side, forward)
    m = np.broadcast_to(np.identity(4, dtype=eye.dtype), eye.shape[:-1] + (4, 4)).copy()
    m[..., 0, :3] = side
    m[..., 1, :3] = up
    m[..., 2, :3] = -forward
    return eye, m


def view_matrices(eye, centre, up) -> np.ndarray:
    """Camera.view_matrix of every row of eye (..., 3) (centre, up: one per
    row or shared)."""
    eye, m = _look_at_rows(eye, centre, up)
    translation = np.broadcast_to(np.identity(4, dtype=eye.dtype), m.shape).copy()
    translation[..., :3, 3] = -eye
    return bmatmul(m, translation)


def view_matrices_inv(eye, centre, up) -> np.ndarray:
    """Camera.view_matrix_inv of every row of eye (..., 3)."""
    eye, m = _look_at_rows(eye, centre, up)
    translation_inv = np.broadcast_to(np.identity(4, dtype=eye.dtype), m.shape).copy()
    translation_inv[..., :3, 3] = eye
    return bmatmul(translation_inv, np.ascontiguousarray(np.swapaxes(m, -1, -2)))


def apply_vec_rows(vectors, matrices) -> np.ndarray:
    """Camera.apply_vec of one direction (or one per row) by matrices
    (..., 4, 4), one result per matrix."""
    v = normalise_rows(_arr(vectors))
    h = to_homogeneous(v, np.zeros((), dtype=v.dtype))
    h = np.broadcast_to(h, np.asarray(matrices).shape[:-2] + (4,))
    return normalise_rows(bmatvec(matrices, h)[..., :3])


class Camera(NamedTuple):
    """Camera matrices (geometry.py:205-278), 4x4 row-major NumPy arrays."""

    view: np.ndarray
    projection: np.ndarray
    viewport: np.ndarray
    world_to_clip: np.ndarray
    world_to_eye_norm: np.ndarray
    world_to_screen: np.ndarray
    view_inv: np.ndarray
    screen_to_world: np.ndarray

    @classmethod
    def create(cls, view, projection, viewport, view_inv=None) -> "Camera":
        view = _arr(view)
        projection = _arr(projection)
        viewport = _arr(viewport)
        if view_inv is None:
            view_inv = lu_inverse(view)
        view_inv = _arr(view_inv)
        if abs(float(projection[3, 3])) <= 1e-8:
            projection_inv = cls.perspective_projection_matrix_inv(projection)
        else:
            projection_inv = cls.orthographic_projection_matrix_inv(projection)
        viewport_inv = cls.viewport_matrix_inv(viewport)
        return cls(
            view=view,
            projection=projection,
            viewport=viewport,
            world_to_clip=matmul(projection, view),
            world_to_eye_norm=np.ascontiguousarray(view_inv.T),
            world_to_screen=matmul(matmul(viewport, projection), view),
            view_inv=view_inv,
            screen_to_world=matmul(matmul(view_inv, projection_inv), viewport_inv),
        )

    @staticmethod
    def apply(points, matrix) -> np.ndarray:
        """Transform homogeneous points (geometry.py:284-315)."""
        return matvec(_arr(matrix), _arr(points))

    @classmethod
    def apply_pos(cls, points, matrix) -> np.ndarray:
        """Transform 3D positions (geometry.py:321-346)."""
        return to_cartesian(cls.apply(to_homogeneous(points), matrix))

    @classmethod
    def apply_vec(cls, vectors, matrix) -> np.ndarray:
        """Transform directions; normalised before and after (geometry.py:352-389)."""
        v = _arr(vectors)
        h = to_homogeneous(normalise(v), np.zeros((), dtype=v.dtype))
        return normalise(cls.apply(h, matrix)[..., :3])

    def to_screen(self, points) -> np.ndarray:
        return normalise_homogeneous(self.apply(points, self.world_to_screen))

    def to_clip(self, points) -> np.ndarray:
        return self.apply(points, self.world_to_clip)

    @staticmethod
    def inv_scale_translation_matrix(mat) -> np.ndarray:
        """Inverse of a scale-then-translate matrix (geometry.py:491-530)."""
        m = _arr(mat)
        one = np.asarray(1.0, dtype=m.dtype)
        scale_inv = np.diag(one / np.diag(m)).astype(m.dtype)
        translation = matmul(scale_inv, m)
        translation_inv = np.identity(4, dtype=m.dtype)
        translation_inv[:3, 3] = -translation[:3, 3]
        return matmul(translation_inv, scale_inv)

    @staticmethod
    def view_matrix(eye, centre, up) -> np.ndarray:
        """lookAt (geometry.py:536-575)."""
        eye = _arr(eye)
        centre = _arr(centre, eye.dtype)
        up = _arr(up, eye.dtype)
        forward = normalise(centre - eye)
        up = normalise(up)
        side = normalise(cross(forward, up))
        up = cross(side, forward)
        m = np.identity(4, dtype=eye.dtype)
        m[0, :3] = side
        m[1, :3] = up
        m[2, :3] = -forward
        translation = np.identity(4, dtype=eye.dtype)
        translation[:3, 3] = -eye
        return matmul(m, translation)

    @staticmethod
    def view_matrix_inv(eye, centre, up) -> np.ndarray:
        """Inverse of lookAt from its parts (geometry.py:581-632)."""
        eye = _arr(eye)
        centre = _arr(centre, eye.dtype)
        up = _arr(up, eye.dtype)
        forward = normalise(centre - eye)
        up = normalise(up)
        side = normalise(cross(forward, up))
        up = cross(side, forward)
        m = np.identity(4, dtype=eye.dtype)
        m[0, :3] = side
        m[1, :3] = up
        m[2, :3] = -forward
        translation_inv = np.identity(4, dtype=eye.dtype)
        translation_inv[:3, 3] = eye
        return matmul(translation_inv, np.ascontiguousarray(m.T))

    @staticmethod
    def perspective_projection_matrix(fovy, aspect, z_near, z_far, dtype=F32) -> np.ndarray:
        """gluPerspective (geometry.py:638-684)."""
        deg = np.asarray(fovy, dtype=dtype)
        rad = deg * np.asarray(np.pi / 180.0, dtype=dtype)
        f = np.asarray(1.0, dtype=dtype) / np.tan(rad / np.asarray(2.0, dtype=dtype))
        aspect = np.asarray(aspect, dtype=dtype)
        z_near = np.asarray(z_near, dtype=dtype)
        z_far = np.asarray(z_far, dtype=dtype)
        p = np.zeros((4, 4), dtype=dtype)
        p[0, 0] = f / aspect
        p[1, 1] = f
        p[2, 2] = (z_far + z_near) / (z_near - z_far)
        p[2, 3] = ((np.asarray(2.0, dtype=dtype) * z_far) * z_near) / (z_near - z_far)
        p[3, 2] = -1.0
        return p

    @classmethod
    def perspective_projection_matrix_inv(cls, mat) -> np.ndarray:
        m = _arr(mat)
        shuffle = np.array((0, 1, 3, 2))
        return cls.inv_scale_translation_matrix(m[:, shuffle])[shuffle, :]

    @staticmethod
    def orthographic_projection_matrix(left, right, bottom, top, z_near, z_far, dtype=F32):
        """glOrtho (geometry.py:720-763)."""
        c = lambda v: np.asarray(v, dtype=dtype)  # noqa: E731
        l_op = np.array([right, top, z_far], dtype=dtype)
        r_op = np.array([left, bottom, z_near], dtype=dtype)
        p = np.zeros((4, 4), dtype=dtype)
        p[0, 0] = c(2) / (c(right) - c(left))
        p[1, 1] = c(2) / (c(top) - c(bottom))
        p[2, 2] = c(-2) / (c(z_far) - c(z_near))
        p[3, 3] = 1
        p[:3, 3] = -(l_op + r_op) / (l_op - r_op)
        return p

    @classmethod
    def orthographic_projection_matrix_inv(cls, mat) -> np.ndarray:
        return cls.inv_scale_translation_matrix(mat)

    @staticmethod
    def viewport_matrix(lowerbound, dimension, depth, dtype=F32) -> np.ndarray:
        """Viewport (geometry.py:813-845)."""
        lb = np.asarray(lowerbound)
        dim = np.asarray(dimension)
        half = (dim / 2).astype(dtype)
        vp = np.identity(4, dtype=dtype)
        vp[:2, 3] = (lb.astype(dtype) + half).astype(dtype)
        vp[0, 0] = half[0]
        vp[1, 1] = half[1]
        d = np.asarray(depth, dtype=dtype) / np.asarray(2, dtype=dtype)
        vp[2, 2] = d
        vp[2, 3] = d
        return vp

    @classmethod
    def viewport_matrix_inv(cls, viewport) -> np.ndarray:
        return cls.inv_scale_translation_matrix(viewport)

    @staticmethod
    def world_to_screen_matrix(width: int, height: int) -> np.ndarray:
        a = np.identity(4, dtype=F32)
        a[0, 0] = 0.5
        a[1, 1] = 0.5
        b = np.eye(4, dtype=F32)
        b[0, 0] = width
        b[1, 1] = height
        c = np.identity(4, dtype=F32)
        c[:2, -1] = 1
        return matmul(matmul(a, b), c)


def compute_normal(triangle_verts) -> np.ndarray:
    t = _arr(triangle_verts)
    n = cross(t[2] - t[0], t[1] - t[0])
    return n / np.sqrt(_sum_sq(n))


def quaternion(rotation_axis, rotation_angle) -> np.ndarray:
    """(w, x, y, z) rotation from an axis and an angle in degrees (geometry.py:909-933)."""
    axis = normalise(_arr(rotation_axis))
    angle = np.asarray(rotation_angle, dtype=axis.dtype) * np.asarray(np.pi / 180, dtype=axis.dtype)
    q = np.zeros(4, dtype=axis.dtype)
    q[0] = np.cos(angle / 2)
    q[1:] = axis * np.sin(angle / 2)
    return q


def quaternion_mul(quatA, quatB) -> np.ndarray:
    """Composition of two (w, x, y, z) quaternions (geometry.py:939-963)."""
    a = _arr(quatA)
    b = _arr(quatB)
    dot = lambda u, v: (u[0] * v[0] + u[1] * v[1]) + u[2] * v[2]  # noqa: E731
    return np.array(
        (
            a[0] * b[0] - dot(a[1:], b[1:]),
            dot(a[:3], b[[1, 0, 3]]) - a[3] * b[2],
            dot(a[[2, 3, 0]], b[:3]) - a[1] * b[3],
            dot(a[[0, 1, 3]], b[[3, 2, 0]]) - a[2] * b[1],
        ),
        dtype=a.dtype,
    )


def rotation_matrix(rotation_axis, rotation_angle) -> np.ndarray:
    """glRotate-style 3x3 rotation, angle in degrees (geometry.py:969-997)."""
    axis = normalise(_arr(rotation_axis))
    angle = np.asarray(rotation_angle, dtype=axis.dtype) * np.asarray(np.pi / 180, dtype=axis.dtype)
    c = np.cos(angle)
    eye = np.identity(3, dtype=axis.dtype)
    return eye * c - np.sin(angle) * cross(axis, eye) + (1 - c) * np.outer(axis, axis)


def transform_matrix_from_rotation(rotation) -> np.ndarray:
    """3x3 matrix of a (w, x, y, z) quaternion (geometry.py:1003-1031)."""
    r = _arr(rotation)
    d = ((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]) + r[3] * r[3]
    s = np.asarray(2.0, dtype=r.dtype) / d
    rs = r[1:] * s
    o = np.outer(r[:3], rs)
    (wx, wy, wz), (xx, xy, xz), (_, yy, yz) = o
    zz = r[3] * rs[2]
    one = np.asarray(1.0, dtype=r.dtype)
    return np.array(
        (
            (one - (yy + zz), xy - wz, xz + wy),
            (xy + wz, one - (xx + zz), yz - wx),
            (xz - wy, yz + wx, one - (xx + yy)),
        ),
        dtype=r.dtype,
    )


Viewport = np.ndarray
View = np.ndarray
Projection = np.ndarray
World2Screen = np.ndarray

__all__ = [
    "Camera",
    "Interpolation",
    "interpolate",
    "normalise",
    "to_homogeneous",
    "normalise_homogeneous",
    "to_cartesian",
    "compute_normal",
    "quaternion",
    "quaternion_mul",
    "rotation_matrix",
    "transform_matrix_from_rotation",
    "lu_inverse",
    "det3",
    "matmul",
    "matvec",
]
