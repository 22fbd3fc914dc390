"""Camera helpers for the draw cull: a column-major view-projection matrix
(the layout src/gfx/fcull.c:20-35 reads) from an eye, a target and a
perspective."""
import numpy as np


def perspective_view(eye, target, fov_deg=70.0, aspect=16 / 9, near=0.1, far=16384.0):
    """float32[16], column-major: projection @ look-at view, y up."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    up = np.array([0.0, 1.0, 0.0])
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = -view[:3, :3] @ eye
    t = 1.0 / np.tan(np.radians(fov_deg) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / aspect, t
    proj[2, 2], proj[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    proj[3, 2] = -1.0
    return (proj @ view).astype(np.float32).T.reshape(16).copy()
