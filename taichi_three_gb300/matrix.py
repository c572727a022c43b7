"""Camera and model matrices (numpy float64) with the names and conventions of
Tina's tina/util/matrix.py: column vectors, right-handed view space looking
down -z, OpenGL clip space.

The projections are the OpenGL ones (glOrtho, glFrustum, gluPerspective) and
the view matrix is gluLookAt's.  Every entry is computed with the operations,
grouped the same way, that give Tina's float64 values bit for bit: the engine
rounds proj @ view to float32, and depth buffers are compared bit for bit.
The `transformations` package that Tina's module imports at load time is not
needed (none of these functions uses it).
"""
import numpy as np


def identity():
    return np.eye(4)


def affine(lin, pos):
    """The 4x4 matrix [lin | pos; 0 0 0 1] (tina/util/matrix.py:8-12)."""
    out = np.zeros((4, 4))
    out[:3, :3] = lin
    out[:3, 3] = pos
    out[3, 3] = 1.0
    return out


def lookat(pos=(0, 0, 0), back=(0, 0, 3), up=(0, 1, 1e-12)):
    """World-to-view matrix of a camera at `pos + back` looking at `pos`
    (tina/util/matrix.py:22-34): the inverse of the camera frame whose
    columns are right, up and -forward, forward = -back / |back|."""
    target = np.array(pos, dtype=float)
    offset = np.array(back, dtype=float)
    forward = -offset
    forward /= np.linalg.norm(forward)
    side = np.cross(forward, np.array(up, dtype=float))
    side /= np.linalg.norm(side)
    frame = np.eye(4)
    frame[:3, 0] = side
    frame[:3, 1] = np.cross(side, forward)
    frame[:3, 2] = -forward
    frame[:3, 3] = target + offset
    return np.linalg.inv(frame)


def ortho(left=-1, right=1, bottom=-1, top=1, near=-100, far=100):
    """glOrtho: the box [left, right] x [bottom, top] x [-near, -far] onto
    the clip cube (tina/util/matrix.py:37-45)."""
    w, h, d = right - left, top - bottom, far - near
    return np.array([[2 / w, 0.0, 0.0, -(right + left) / w],
                     [0.0, 2 / h, 0.0, -(top + bottom) / h],
                     [0.0, 0.0, -2 / d, -(far + near) / d],
                     [0.0, 0.0, 0.0, 1.0]])


def frustum(left=-1, right=1, bottom=-1, top=1, near=1, far=100):
    """glFrustum: the view pyramid through [left, right] x [bottom, top] at
    distance `near`, cut at `far` (tina/util/matrix.py:48-58)."""
    w, h, d = right - left, top - bottom, far - near
    return np.array([[2 * near / w, 0.0, (right + left) / w, 0.0],
                     [0.0, 2 * near / h, (top + bottom) / h, 0.0],
                     [0.0, 0.0, -(far + near) / d, -2 * far * near / d],
                     [0.0, 0.0, -1.0, 0.0]])


def orthogonal(size=1, aspect=1, near=-100, far=100):
    """ortho of half-height `size` and half-width `size * aspect`."""
    return ortho(-(size * aspect), size * aspect, -size, size, near, far)


def perspective(fov=60, aspect=1, near=0.05, far=500):
    """gluPerspective: vertical field of view `fov` degrees
    (tina/util/matrix.py:66-69)."""
    half = np.tan(np.radians(fov) / 2)
    x, y = near * (half * aspect), near * half
    return frustum(-x, x, -y, y, near, far)


def scale(factor):
    """Scaling by `factor` (a number or three)."""
    return affine(np.eye(3) * np.array(factor), np.zeros(3))


def translate(offset):
    """Translation by `offset` (a number or three)."""
    return affine(np.eye(3), np.array(offset) * np.ones(3))


def quaternion(q):
    """Rotation of the unit quaternion (x, y, z, w) (tina/util/matrix.py:81-92)."""
    x, y, z, w = q[0], q[1], q[2], q[3]
    return affine(np.array([
        [1.0 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (w * y + x * z)],
        [2 * (x * y + w * z), 1.0 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1.0 - 2 * (x * x + y * y)]]), np.zeros(3))


def _axis_rotation(axis, angle):
    c, s = np.cos(angle), np.sin(angle)
    i, j = [(1, 2), (0, 2), (0, 1)][axis]
    r = np.eye(3)
    r[i, i], r[j, j] = c, c
    # the y rotation turns z into x: its sine terms swap signs
    r[i, j], r[j, i] = (s, -s) if axis == 1 else (-s, s)
    return r


def eularXYZ(theta):
    """Rotation about x by theta[0], then y by theta[1], then z by theta[2]:
    R_z @ R_y @ R_x (tina/util/matrix.py:96-104)."""
    return affine(_axis_rotation(2, theta[2]) @ _axis_rotation(1, theta[1]) @ _axis_rotation(0, theta[0]),
                  np.zeros(3))


def orbit_camera(theta=0.0, phi=0.0, radius=3.0, center=(0, 0, 0)):
    """Headless stand-in for tina.Control's default camera (tina/util/control.py:13-15,
    102-113): a camera at distance `radius` from `center`, rotated by altitude
    `theta` and longitude `phi` (radians), looking at the centre."""
    center = np.asarray(center, dtype=float)
    back = np.array([np.sin(phi) * np.cos(theta), np.sin(theta), np.cos(phi) * np.cos(theta)])
    return lookat(center, back * radius)
