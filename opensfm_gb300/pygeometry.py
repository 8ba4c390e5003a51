"""Camera and Pose types with the attribute names of opensfm.pygeometry.

The bundle adjuster takes these objects exactly where the reference's pybind
module takes geometry::Camera / geometry::Pose
(opensfm/src/lib/geometry/pygeometry.pyi:67-299).  Camera parameter vectors
follow geometry::Camera (geometry/src/camera.cc:11-172); Pose stores the
world-to-camera rotation (angle-axis) and translation like geometry::Pose
(geometry/pose.h).
"""
from __future__ import annotations

import copy
import enum

import numpy as np

from . import synthetic as _syn
from .scene import (BROWN, DUAL, FISHEYE, FISHEYE62, FISHEYE624, FISHEYE_OPENCV, PERSPECTIVE, RADIAL,
                    SIMPLE_RADIAL, SPHERICAL)


class CameraParameters(enum.IntEnum):
    transition = 0
    k1 = 1
    k2 = 2
    k3 = 3
    k4 = 4
    k5 = 5
    k6 = 6
    p1 = 7
    p2 = 8
    focal = 9
    aspect_ratio = 10
    cx = 11
    cy = 12
    s0 = 13
    s1 = 14
    s2 = 15
    s3 = 16
    none = 17


_P = CameraParameters
_TYPES = {
    PERSPECTIVE: [_P.k1, _P.k2, _P.focal],
    BROWN: [_P.k1, _P.k2, _P.k3, _P.p1, _P.p2, _P.focal, _P.aspect_ratio, _P.cx, _P.cy],
    FISHEYE: [_P.k1, _P.k2, _P.focal],
    FISHEYE_OPENCV: [_P.k1, _P.k2, _P.k3, _P.k4, _P.focal, _P.aspect_ratio, _P.cx, _P.cy],
    FISHEYE62: [_P.k1, _P.k2, _P.k3, _P.k4, _P.k5, _P.k6, _P.p1, _P.p2, _P.focal, _P.aspect_ratio, _P.cx, _P.cy],
    FISHEYE624: [_P.k1, _P.k2, _P.k3, _P.k4, _P.k5, _P.k6, _P.p1, _P.p2, _P.s0, _P.s1, _P.s2, _P.s3, _P.focal,
                 _P.aspect_ratio, _P.cx, _P.cy],
    SPHERICAL: [_P.none],
    DUAL: [_P.transition, _P.k1, _P.k2, _P.focal],
    RADIAL: [_P.k1, _P.k2, _P.focal, _P.aspect_ratio, _P.cx, _P.cy],
    SIMPLE_RADIAL: [_P.k1, _P.focal, _P.aspect_ratio, _P.cx, _P.cy],
}
_NAMES = {PERSPECTIVE: "perspective", BROWN: "brown", FISHEYE: "fisheye", FISHEYE_OPENCV: "fisheye_opencv",
          FISHEYE62: "fisheye62", FISHEYE624: "fisheye624", SPHERICAL: "spherical", DUAL: "dual",
          RADIAL: "radial", SIMPLE_RADIAL: "simple_radial"}


class Camera:
    """geometry::Camera: a projection model and its parameter vector."""

    def __init__(self, model: int = PERSPECTIVE, values=None):
        self.model = int(model)
        self._values = np.zeros(len(_TYPES[self.model])) if values is None else np.asarray(values, float).copy()
        self.id = ""
        self.width = 1
        self.height = 1

    # factories (geometry/src/camera.cc:11-172)
    @staticmethod
    def create_perspective(focal, k1, k2):
        return Camera(PERSPECTIVE, [k1, k2, focal])

    @staticmethod
    def create_brown(focal, aspect_ratio, principal_point, distortion):
        d = np.asarray(distortion, float)
        if d.size != 5:
            raise RuntimeError("Invalid distortion coefficients size")
        return Camera(BROWN, list(d) + [focal, aspect_ratio, principal_point[0], principal_point[1]])

    @staticmethod
    def create_fisheye(focal, k1, k2):
        return Camera(FISHEYE, [k1, k2, focal])

    @staticmethod
    def create_fisheye_opencv(focal, aspect_ratio, principal_point, distortion):
        d = np.asarray(distortion, float)
        if d.size != 4:
            raise RuntimeError("Invalid distortion coefficients size")
        return Camera(FISHEYE_OPENCV, list(d) + [focal, aspect_ratio, principal_point[0], principal_point[1]])

    @staticmethod
    def create_fisheye62(focal, aspect_ratio, principal_point, distortion):
        d = np.asarray(distortion, float)
        if d.size != 8:
            raise RuntimeError("Invalid distortion coefficients size")
        return Camera(FISHEYE62, list(d) + [focal, aspect_ratio, principal_point[0], principal_point[1]])

    @staticmethod
    def create_fisheye624(focal, aspect_ratio, principal_point, distortion):
        d = np.asarray(distortion, float)
        if d.size != 12:
            raise RuntimeError("Invalid distortion coefficients size")
        return Camera(FISHEYE624, list(d) + [focal, aspect_ratio, principal_point[0], principal_point[1]])

    @staticmethod
    def create_dual(transition, focal, k1, k2):
        return Camera(DUAL, [transition, k1, k2, focal])

    @staticmethod
    def create_spherical():
        return Camera(SPHERICAL, [0.0])

    @staticmethod
    def create_radial(focal, aspect_ratio, principal_point, distortion):
        return Camera(RADIAL, [distortion[0], distortion[1], focal, aspect_ratio, principal_point[0],
                               principal_point[1]])

    @staticmethod
    def create_simple_radial(focal, aspect_ratio, principal_point, k1):
        return Camera(SIMPLE_RADIAL, [k1, focal, aspect_ratio, principal_point[0], principal_point[1]])

    # parameters
    def get_parameters_types(self):
        return list(_TYPES[self.model])

    def get_parameters_values(self) -> np.ndarray:
        return self._values.copy()

    def set_parameters_values(self, values) -> None:
        v = np.asarray(values, float)
        if v.size != self._values.size:
            raise RuntimeError("Invalid parameter vector size")
        self._values = v.copy()

    def get_parameters_map(self):
        return dict(zip(_TYPES[self.model], self._values))

    def _get(self, p):
        types = _TYPES[self.model]
        if p not in types:
            raise RuntimeError("Unknown parameter for this camera model")
        return float(self._values[types.index(p)])

    def set_parameter_value(self, p, value: float) -> None:
        types = _TYPES[self.model]
        if p not in types:
            raise RuntimeError("Unknown parameter for this camera model")
        self._values[types.index(p)] = value

    @property
    def projection_type(self) -> str:
        return _NAMES[self.model]

    focal = property(lambda s: s._get(_P.focal), lambda s, v: s.set_parameter_value(_P.focal, v))
    aspect_ratio = property(lambda s: s._get(_P.aspect_ratio),
                            lambda s, v: s.set_parameter_value(_P.aspect_ratio, v))
    transition = property(lambda s: s._get(_P.transition), lambda s, v: s.set_parameter_value(_P.transition, v))
    k1 = property(lambda s: s._get(_P.k1))
    k2 = property(lambda s: s._get(_P.k2))
    k3 = property(lambda s: s._get(_P.k3))
    k4 = property(lambda s: s._get(_P.k4))
    k5 = property(lambda s: s._get(_P.k5))
    k6 = property(lambda s: s._get(_P.k6))
    p1 = property(lambda s: s._get(_P.p1))
    p2 = property(lambda s: s._get(_P.p2))
    s0 = property(lambda s: s._get(_P.s0))
    s1 = property(lambda s: s._get(_P.s1))
    s2 = property(lambda s: s._get(_P.s2))
    s3 = property(lambda s: s._get(_P.s3))

    @property
    def principal_point(self) -> np.ndarray:
        return np.array([self._get(_P.cx), self._get(_P.cy)])

    @principal_point.setter
    def principal_point(self, pp) -> None:
        self.set_parameter_value(_P.cx, pp[0])
        self.set_parameter_value(_P.cy, pp[1])

    def project(self, point) -> np.ndarray:
        return _syn.project(self.model, self._values, np.asarray(point, float))

    def project_many(self, points) -> np.ndarray:
        p = np.asarray(points, float)
        return _syn.project(self.model, np.broadcast_to(self._values, (len(p), self._values.size)), p)

    def bearing(self, point, iterations: int = 20) -> np.ndarray:
        """Camera::Bearing: the unit camera-frame direction that projects to
        the normalized image point.  Spherical cameras invert their
        longitude/latitude map directly; the other models solve project((x,
        y, 1)) = point by Gauss-Newton with a central-difference Jacobian,
        from the point itself divided by the focal length (the reference's
        models invert their distortion by Newton steps too)."""
        u = np.asarray(point, float)
        if self.model == SPHERICAL:
            lon, lat = 2 * np.pi * u[0], -2 * np.pi * u[1]
            return np.array([np.cos(lat) * np.sin(lon), -np.sin(lat), np.cos(lat) * np.cos(lon)])
        f = float(self._get(_P.focal)) if _P.focal in self.get_parameters_types() else 1.0
        xy = u / (f if f else 1.0)
        h = 1e-7
        for _ in range(iterations):
            r = self.project(np.r_[xy, 1.0]) - u
            if np.abs(r).max() < 1e-14:
                break
            J = np.empty((2, 2))
            for k in range(2):
                d = np.zeros(2)
                d[k] = h
                J[:, k] = (self.project(np.r_[xy + d, 1.0]) - self.project(np.r_[xy - d, 1.0])) / (2 * h)
            xy = xy - np.linalg.solve(J, r)
        b = np.r_[xy, 1.0]
        return b / np.linalg.norm(b)

    def __copy__(self):
        c = Camera(self.model, self._values)
        c.id, c.width, c.height = self.id, self.width, self.height
        return c

    def __deepcopy__(self, memo):
        return self.__copy__()


class Similarity:
    """geometry::Similarity (geometry/similarity.h): x -> scale R x +
    translation, R given as an angle-axis ``rotation``; the camera bias of
    the bundle adjuster (bundle/data/bias.h)."""

    def __init__(self, rotation=None, translation=None, scale: float = 1.0):
        self.rotation = np.zeros(3) if rotation is None else np.asarray(rotation, float).copy()
        self.translation = np.zeros(3) if translation is None else np.asarray(translation, float).copy()
        self.scale = float(scale)

    def get_rotation_matrix(self) -> np.ndarray:
        return _syn.rotation_matrix(self.rotation)

    def transform(self, point) -> np.ndarray:
        return self.scale * (self.get_rotation_matrix() @ np.asarray(point, float)) + self.translation

    def is_valid(self) -> bool:
        return bool(np.all(np.isfinite(self.rotation)) and np.all(np.isfinite(self.translation))
                    and np.isfinite(self.scale))


class Pose:
    """geometry::Pose: x_cam = R x_world + t, R given as an angle-axis.

    ``Pose(rotation, translation)`` takes the world-to-camera angle-axis and
    translation, as the reference constructor does."""

    def __init__(self, rotation=None, translation=None):
        self.rotation = np.zeros(3) if rotation is None else np.asarray(rotation, float).copy()
        self.translation = np.zeros(3) if translation is None else np.asarray(translation, float).copy()

    def get_rotation_matrix(self) -> np.ndarray:
        return _syn.rotation_matrix(self.rotation)

    get_R_world_to_cam = get_rotation_matrix

    def get_R_cam_to_world(self) -> np.ndarray:
        return self.get_rotation_matrix().T

    def get_R_world_to_cam_min(self) -> np.ndarray:
        return self.rotation.copy()

    def get_R_cam_to_world_min(self) -> np.ndarray:
        return -self.rotation

    def get_t_world_to_cam(self) -> np.ndarray:
        return self.translation.copy()

    def get_origin(self) -> np.ndarray:
        return -self.get_rotation_matrix().T @ self.translation

    def set_origin(self, origin) -> None:
        self.translation = -self.get_rotation_matrix() @ np.asarray(origin, float)

    def set_rotation_matrix(self, R) -> None:
        self.rotation = _syn.rotation_vector(np.asarray(R, float))

    def transform(self, point) -> np.ndarray:
        return self.get_rotation_matrix() @ np.asarray(point, float) + self.translation

    def transform_inverse(self, point) -> np.ndarray:
        return self.get_rotation_matrix().T @ (np.asarray(point, float) - self.translation)

    def inverse(self) -> "Pose":
        R = self.get_rotation_matrix().T
        p = Pose()
        p.set_rotation_matrix(R)
        p.translation = -R @ self.translation
        return p

    def compose(self, other: "Pose") -> "Pose":
        R1 = self.get_rotation_matrix()
        p = Pose()
        p.set_rotation_matrix(R1 @ other.get_rotation_matrix())
        p.translation = R1 @ other.translation + self.translation
        return p

    # bundle::Pose data layout (camera-to-world): [rx ry rz | origin]
    def ba_data(self) -> np.ndarray:
        return np.concatenate([-self.rotation, self.get_origin()])

    @staticmethod
    def from_ba_data(data) -> "Pose":
        d = np.asarray(data, float)
        p = Pose(-d[:3])
        p.set_origin(d[3:6])
        return p

    def __copy__(self):
        return Pose(self.rotation, self.translation)

    def __deepcopy__(self, memo):
        return self.__copy__()

    def __repr__(self) -> str:
        return f"Pose(rotation={self.rotation.tolist()}, translation={self.translation.tolist()})"


__all__ = ["Camera", "CameraParameters", "Pose", "Similarity"]
_ = copy
