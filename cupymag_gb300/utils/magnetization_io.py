"""Magnetisation files and initial state (cupymag/utils/magnetization_io.py:21-124).

``write_array``/``read_array`` use HDF5 (dataset "data") when h5py is
installed and ``.npy`` otherwise; ``read_array`` returns None (with the
reference's message) on a missing name or a shape other than (nDOF, 3).
``initialize_m`` builds uniform m from ``initial_magnetization`` (normalised)
or restarts from a file, then zeroes the defect DOFs.
"""
from pathlib import Path

import numpy as np

try:  # optional
    import h5py  # type: ignore
except Exception:  # pragma: no cover
    h5py = None


def _as_numpy(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def write_array(array, filename):
    filename = Path(filename)
    data = _as_numpy(array)
    if h5py is not None and filename.suffix in (".h5", ""):
        filename = filename.with_suffix(".h5")
        with h5py.File(filename, "w") as f:
            f.create_dataset("data", data=data, compression="gzip", compression_opts=6)
            f.attrs["shape"] = data.shape
            f.attrs["dtype"] = str(data.dtype)
        return filename
    filename = filename.with_suffix(".npy")
    np.save(filename, data)
    return filename


def read_array(filename, nDOF):
    if filename is None:
        print("Initial magnetization file not found, start with uniform magnetization.")
        return None
    filename = Path(filename)
    if filename.suffix == ".npy" or h5py is None:
        p = filename if filename.suffix == ".npy" else filename.with_suffix(".npy")
        data = np.load(p)
    else:
        with h5py.File(filename.with_suffix(".h5"), "r") as f:
            data = f["data"][:]
    if data.shape != (nDOF, 3):
        print(f"Initial magnetization shape mismatch: expected ({nDOF}, 3), got {data.shape}.")
        print("Start with uniform magnetization.")
        return None
    return data


def initialize_m(restart_m, restart, initial_m, nDOF, DefDOF):
    m = read_array(restart_m, nDOF) if restart else None
    if m is None:
        if initial_m is None:
            v = np.array([1.0, 0.0, 0.0])
        else:
            v = np.array(initial_m, dtype=np.float64)
            nrm = np.linalg.norm(v)
            if nrm > 0:
                v = v / nrm
            else:
                raise ValueError("Initial magnetization vector cannot be zero.")
        m = np.empty((nDOF, 3))
        m[:] = v[None, :]
    m = np.array(m, dtype=np.float64)
    m[np.asarray(DefDOF, dtype=np.int64), :] = 0.0
    return m


def seeded_initial_m(nDOF, DefDOF, seed, sigma=1e-3, direction=(1.0, 0.0, 0.0)):
    """normalise(direction + N(0, sigma)) with numpy.random.default_rng(seed); defect DOFs zero."""
    rng = np.random.default_rng(seed)
    m = np.asarray(direction, dtype=np.float64)[None, :] + rng.normal(0.0, sigma, size=(nDOF, 3))
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    m[np.asarray(DefDOF, dtype=np.int64), :] = 0.0
    return m
