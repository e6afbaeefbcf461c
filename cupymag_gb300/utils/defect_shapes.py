"""Non-magnetic defect indicator functions (cupymag/utils/defect_shapes.py:21-161).

Registry of shapes; each ``shape_fn(rel_coords)`` returns True where the
point (relative to the defect centre) lies inside.  RotatedEllipsoid uses
Q = R diag(1/a^2, 1/b^2, 1/c^2) R^T (defect_shapes.py:113-134).
"""
import numpy as np

_REGISTRY = {}


def register_shape(name):
    def deco(fn):
        _REGISTRY[name] = fn
        return fn
    return deco


@register_shape("Sphere")
def _sphere(params):
    R = float(np.ravel(params)[0])
    R2 = R * R
    return lambda rel: np.sum(np.atleast_2d(rel) ** 2, axis=1) < R2


@register_shape("Ellipsoid")
def _ellipsoid(params):
    a, b, c = (float(v) for v in params)
    inv2 = np.array([1.0 / a ** 2, 1.0 / b ** 2, 1.0 / c ** 2])
    return lambda rel: np.sum(np.atleast_2d(rel) ** 2 * inv2[None, :], axis=1) < 1.0


@register_shape("RotatedEllipsoid")
def _rotated(params):
    abc, R = params
    a, b, c = (float(v) for v in abc)
    R = np.asarray(R, dtype=float)
    Q = R @ np.diag([1.0 / a ** 2, 1.0 / b ** 2, 1.0 / c ** 2]) @ R.T

    def fn(rel):
        rel = np.atleast_2d(rel)
        return np.sum((rel @ Q) * rel, axis=1) < 1.0
    return fn


def get_supported_shapes():
    return list(_REGISTRY)


def get_defect_shape_function(defect_shape, shape_params):
    if defect_shape not in _REGISTRY:
        raise NotImplementedError(f"Defect shape '{defect_shape}' is not supported. "
                                  f"Supported shapes: {get_supported_shapes()}")
    return _REGISTRY[defect_shape](shape_params)
