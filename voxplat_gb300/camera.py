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


def camera(eye, target, width, height, fov_deg=70.0, near=0.1, far=16384.0):
    """The reference camera's matrices (view = rotation x translation):
    projection, view_rotation, view_translation, view_projection,
    inv_proj_view_rot and proj_view_rot (float32[16] column-major each),
    far plane and viewport, as vp_camera wants them."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    up = np.array([0.0, 1.0, 0.0])
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    rot = np.eye(4)
    rot[0, :3], rot[1, :3], rot[2, :3] = s, u, -f
    tra = np.eye(4)
    tra[:3, 3] = -eye
    t = 1.0 / np.tan(np.radians(fov_deg) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / (width / height), t
    proj[2, 2], proj[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    proj[3, 2] = -1.0
    pvr = proj @ rot

    def cm(m):
        return m.astype(np.float32).T.reshape(16).copy()

    return {"projection": cm(proj), "view_rotation": cm(rot), "view_translation": cm(tra),
            "view_projection": cm(proj @ rot @ tra), "inv_proj_view_rot": cm(np.linalg.inv(pvr)),
            "proj_view_rot": cm(pvr), "far_plane": float(far), "width": int(width), "height": int(height)}
