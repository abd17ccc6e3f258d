"""The steering STATE record and helpers that fill it the way iVR's client does.

``IvrState`` has the layout of ``STATE`` (connection.h:9-18, 184 bytes): the
per-frame message the reference's client sends and the server renders from.
``orbit_state`` fills it the way the client's ``display()`` does
(ivrclient.c:536-569): a GL model-view matrix that looks at the origin from
distance 5, a ``gluPerspective`` projection, and the view-volume extents of
``getfrustum`` (mathutil.h:166-175).  Matrices are GL column-major, as on the
wire.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

NO_CLIP = 1.0e30  # a newconst this large never shrinks the volume box


class IvrState(ctypes.Structure):
    """``STATE`` (connection.h:9-18)."""

    _fields_ = [
        ("finish", ctypes.c_int),
        ("winwidth", ctypes.c_int),
        ("winheight", ctypes.c_int),
        ("alpha", ctypes.c_float),
        ("newconst", ctypes.c_float * 6),
        ("vv", ctypes.c_float * 4),
        ("mvm", ctypes.c_float * 16),
        ("pm", ctypes.c_float * 16),
    ]

    def as_dict(self) -> dict:
        return {
            "finish": self.finish,
            "winwidth": self.winwidth,
            "winheight": self.winheight,
            "alpha": self.alpha,
            "newconst": list(self.newconst),
            "vv": list(self.vv),
            "mvm": list(self.mvm),
            "pm": list(self.pm),
        }

    @classmethod
    def from_dict(cls, d: dict) -> "IvrState":
        s = cls()
        s.finish = int(d.get("finish", 0))
        s.winwidth = int(d["winwidth"])
        s.winheight = int(d["winheight"])
        s.alpha = float(d["alpha"])
        for name, n in (("newconst", 6), ("vv", 4), ("mvm", 16), ("pm", 16)):
            arr = getattr(s, name)
            vals = d[name]
            for i in range(n):
                arr[i] = float(vals[i])
        return s

    def to_bytes(self) -> bytes:
        return ctypes.string_at(ctypes.addressof(self), ctypes.sizeof(self))

    @classmethod
    def from_bytes(cls, b: bytes) -> "IvrState":
        if len(b) != ctypes.sizeof(cls):
            raise ValueError(f"STATE is {ctypes.sizeof(cls)} bytes, got {len(b)}")
        s = cls()
        ctypes.memmove(ctypes.addressof(s), b, len(b))
        return s


assert ctypes.sizeof(IvrState) == 184


def _lookat(eye, center, up) -> np.ndarray:
    """gluLookAt as a row-major 4x4 (float64)."""
    eye, center, up = (np.asarray(v, dtype=np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    u = up / np.linalg.norm(up)
    s = np.cross(f, u)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    t = np.eye(4)
    t[:3, 3] = -eye
    return m @ t


def _perspective(fovy_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """gluPerspective as a row-major 4x4 (float64)."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[2, 3] = 2.0 * far * near / (near - far)
    m[3, 2] = -1.0
    return m


def frustum_vv(fovy_deg: float, aspect: float) -> list:
    """getfrustum (mathutil.h:166-175): extents of the view plane at the
    eye distance 5 that rays are generated on."""
    fovy = np.float32(math.pi / 180.0 * np.float32(fovy_deg))
    t = np.float32(math.tan(float(np.float32(fovy / np.float32(2.0)))) * 5.0)
    b = -t
    return [float(np.float32(aspect) * b), float(np.float32(aspect) * t), float(b), float(t)]


def orbit_state(az_deg: float, el_deg: float, width: int, height: int, fovy: float = 30.0,
                alpha: float = 1.0, dist: float = 5.0, clip=None) -> IvrState:
    """STATE for a camera at distance ``dist`` on the sphere direction given
    by azimuth/elevation (degrees), looking at the volume centre, ``fovy``
    degrees of vertical field of view.  ``clip``: 6 plane constants
    (``newconst``; -x,+x,-y,+y,-z,+z faces), default none."""
    az, el = math.radians(az_deg), math.radians(el_deg)
    direction = np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
    mvm = _lookat(dist * direction, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    aspect = width / height
    pm = _perspective(fovy, aspect, 0.1, 100.0)
    s = IvrState()
    s.finish = 0
    s.winwidth = int(width)
    s.winheight = int(height)
    s.alpha = float(alpha)
    for i, c in enumerate(clip if clip is not None else [NO_CLIP] * 6):
        s.newconst[i] = float(c)
    for i, v in enumerate(frustum_vv(fovy, aspect)):
        s.vv[i] = v
    for i, v in enumerate(mvm.astype(np.float32).T.reshape(-1)):
        s.mvm[i] = float(v)
    for i, v in enumerate(pm.astype(np.float32).T.reshape(-1)):
        s.pm[i] = float(v)
    return s
