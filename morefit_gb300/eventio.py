"""On-disk event input.

The reference reads events from a ROOT TTree, one branch per dimension
(``load_event_vector``, include/eventvector.hh:297-332: dimension names,
optional branch names, ``max_event``). ROOT files are not readable here;
the same call reads NumPy files:

* ``.npz``: one 1-D array per branch (key = branch name);
* ``.npy`` with a structured dtype: one field per branch;
* ``.npy`` with a 2-D array (ncols, n): the columns of an SoA block, named
  by ``columns`` (default: the dimension names, in order).

``load_event_vector`` returns the host SoA block (ndims, n) in FP64.
``upload_event_file`` puts the columns straight into device memory: for a
C-ordered 2-D ``.npy`` it streams the file through page-locked staging
chunks (``mf_events_load_file``: the read of one chunk overlaps the copy of
the previous one) without a host copy of the whole block; other layouts are
read on the host and uploaded.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _lib as L
from .backend import CUDABackend, DeviceColumns


def _branches(dimensions, branchnames):
    branches = list(dimensions) if not branchnames else list(branchnames)
    if len(branches) != len(dimensions):
        raise ValueError("one branch name per dimension")
    return branches


def _npy_header(path: Path):
    """(shape, fortran_order, dtype, data offset) of a .npy file."""
    with open(path, "rb") as f:
        version = np.lib.format.read_magic(f)
        if version == (1, 0):
            shape, fortran, dtype = np.lib.format.read_array_header_1_0(f)
        else:
            shape, fortran, dtype = np.lib.format.read_array_header_2_0(f)
        return shape, fortran, dtype, f.tell()


def load_event_vector(filename, dimensions, branchnames=None, max_event: int = -1, columns=None) -> np.ndarray:
    """Events (ndims, n) in FP64 from a .npz / .npy file (the reference's
    load_event_vector with NumPy files in place of a ROOT tree)."""
    path = Path(filename)
    branches = _branches(dimensions, branchnames)
    if path.suffix == ".npz":
        with np.load(path) as z:
            missing = [b for b in branches if b not in z.files]
            if missing:
                raise KeyError(f"branches {missing} not in {path}")
            cols = [np.asarray(z[b], dtype=np.float64) for b in branches]
    elif path.suffix == ".npy":
        a = np.load(path, mmap_mode="r")
        if a.dtype.names:
            missing = [b for b in branches if b not in a.dtype.names]
            if missing:
                raise KeyError(f"branches {missing} not in {path}")
            cols = [np.asarray(a[b], dtype=np.float64) for b in branches]
        else:
            if a.ndim != 2:
                raise ValueError(f"{path}: expected a 2-D (columns, events) array")
            names = list(columns) if columns is not None else list(dimensions)
            if len(names) != a.shape[0]:
                raise ValueError(f"{path}: {a.shape[0]} columns, {len(names)} column names")
            missing = [b for b in branches if b not in names]
            if missing:
                raise KeyError(f"branches {missing} not in {path}")
            cols = [np.asarray(a[names.index(b)], dtype=np.float64) for b in branches]
    else:
        raise ValueError(f"unsupported event file {path} (.npz or .npy)")
    n = len(cols[0]) if cols else 0
    if max_event > 0 and max_event < n:
        n = max_event
    return np.ascontiguousarray(np.vstack([c[:n] for c in cols]))


def upload_event_file(backend: CUDABackend, filename, dimensions, branchnames=None, max_event: int = -1,
                      columns=None, elem: int = L.MF_F64) -> DeviceColumns:
    """The events of `filename` as a device block (columns in dimension
    order, element type `elem`). A C-ordered 2-D .npy of FP64 or FP32 values
    is streamed from disk to the device."""
    path = Path(filename)
    branches = _branches(dimensions, branchnames)
    out = DeviceColumns(backend, elem)
    if path.suffix == ".npy":
        shape, fortran, dtype, offset = _npy_header(path)
        if len(shape) == 2 and not fortran and dtype.names is None and dtype in (np.float64, np.float32) \
                and dtype.isnative:
            names = list(columns) if columns is not None else list(dimensions)
            if len(names) != shape[0]:
                raise ValueError(f"{path}: {shape[0]} columns, {len(names)} column names")
            missing = [b for b in branches if b not in names]
            if missing:
                raise KeyError(f"branches {missing} not in {path}")
            n = shape[1] if not (0 < max_event < shape[1]) else max_event
            out.ensure(len(branches), n)
            cols = (C.c_uint32 * max(1, len(branches)))(*[names.index(b) for b in branches])
            L.check(L.lib.mf_events_load_file(out.buf, elem, out.stride, str(path).encode(), offset,
                                              L.MF_F64 if dtype == np.float64 else L.MF_F32, shape[1],
                                              len(branches), cols, n))
            return out
    ev = load_event_vector(path, dimensions, branchnames, max_event, columns)
    out.upload(ev)
    return out


def save_event_vector(filename, events: np.ndarray) -> None:
    """Writes an SoA block (ncols, n) as a 2-D .npy file that
    upload_event_file streams."""
    np.save(filename, np.ascontiguousarray(events))
