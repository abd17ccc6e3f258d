"""CPU: the STATE record and the view helpers."""
import ctypes

import numpy as np

from ivr_gb300.state import IvrState, frustum_vv, orbit_state


def test_state_layout():
    assert ctypes.sizeof(IvrState) == 184  # connection.h:9-18
    assert IvrState.newconst.offset == 16 and IvrState.vv.offset == 40
    assert IvrState.mvm.offset == 56 and IvrState.pm.offset == 120


def test_state_roundtrip():
    s = orbit_state(33, -12, 320, 200, fovy=30, alpha=0.7)
    b = s.to_bytes()
    t = IvrState.from_bytes(b)
    assert t.to_bytes() == b
    assert IvrState.from_dict(s.as_dict()).to_bytes() == b


def test_orbit_looks_at_origin_from_distance_5():
    s = orbit_state(40, 20, 64, 64)
    m = np.array(list(s.mvm), np.float64).reshape(4, 4).T  # column-major
    eye = -m[:3, :3].T @ m[:3, 3]
    assert abs(np.linalg.norm(eye) - 5.0) < 1e-5
    assert abs(m[2, 3] + 5.0) < 1e-5


def test_frustum_matches_fov():
    l, r, b, t = frustum_vv(30.0, 2.0)
    assert abs(t - 5 * np.tan(np.radians(15))) < 1e-5 and abs(r - 2 * t) < 1e-5 and l == -r and b == -t
